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
// NCA. One warp per task (a box's outgoing or incoming block: rows, cols,
// tolerance), tasks taken from an atomic counter. The steps are the host's
// aca_core in the same order: pivot search with ties to the lowest index,
// the rank-1 updates element by element in the same operand order, the
// norm estimate and the stopping rules. Norms and dot products are warp
// reductions (another summation order than the host's loop), so a stopping
// decision taken within rounding of its threshold can differ. A task whose
// rank would pass the scratch's rank capacity is marked and the host redoes
// it. Every loop is bounded by the task's sizes; nothing waits on another
// thread beyond __syncwarp.

#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <string>
#include <vector>

#include "ls_internal.h"

namespace lsg {

namespace {

constexpr int kSeriesG = 15;                 // FarFieldInteraction.hpp:55
constexpr int kTerms = 2 * kSeriesG + 1;
constexpr int kTableKeys = 128;              // keys (threads) per block of the table kernel
constexpr int kNcaWarpsPerBlock = 4;
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

__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}

// First index of the largest |v| among the unused ones, 0 when all are used.
__device__ int warp_argmax(const double2* v, const unsigned char* used, int n, int lane) {
  double best = -1.0;
  int bi = INT_MAX;
  for (int k = lane; k < n; k += 32) {
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

__device__ __forceinline__ double warp_norm(const double2* v, int n, int lane) {
  double s = 0.0;
  for (int k = lane; k < n; k += 32) s += v[k].x * v[k].x + v[k].y * v[k].y;
  return sqrt(warp_sum(s));
}

// sum_k conj(a_k) b_k
__device__ __forceinline__ double2 warp_cdot(const double2* a, const double2* b, int n, int lane) {
  double sr = 0.0, si = 0.0;
  for (int k = lane; k < n; k += 32) {
    const double x = a[k].x, y = a[k].y, c = b[k].x, d = b[k].y;
    sr += x * c + y * d;
    si += x * d - y * c;
  }
  return make_double2(warp_sum(sr), warp_sum(si));
}

// as_row: out[k] = K(rows[fixed], cols[k]), k < n2; else out[k] = K(rows[k], cols[fixed]), k < n1.
__device__ __forceinline__ void fetch(const NcaGeomDev& g, const int* __restrict__ rows,
                                      const int* __restrict__ cols, int n1, int n2, bool as_row, int fixed,
                                      double2* __restrict__ out, int lane) {
  if (as_row) {
    const int i = rows[fixed];
#pragma unroll 4
    for (int k = lane; k < n2; k += 32) out[k] = far_entry(g, i, cols[k]);
  } else {
    const int j = cols[fixed];
#pragma unroll 4
    for (int k = lane; k < n1; k += 32) out[k] = far_entry(g, rows[k], j);
  }
}

// One NCA task by one warp. The first vector fetched lives on domain D1
// (columns when the block has fewer rows than columns, rows otherwise),
// the second on D2; V holds the normalised D1 vectors, U the D2 ones.
__device__ void aca_task(const NcaGeomDev& g, const NcaTask& tk, const int* idx, double eps, double2* scr,
                         unsigned char* used, int* piv, int* rank_out, int* status_out, double2* coef, int lane) {
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
  for (int k = lane; k < d1 + d2; k += 32) used[k] = 0;
  __syncwarp();
  int i1 = 0, i2 = 0, l = 0;
  for (; l < d2; ++l) {
    i2 = l;
    __syncwarp();  // every lane has read p[i1] before p is refetched
    fetch(g, rows, cols, n1, n2, rowfirst, i2, p, lane);
    __syncwarp();
    i1 = warp_argmax(p, used1, d1, lane);
    if (cmag(p[i1]) > eps) break;
  }
  if (l == d2) {
    if (lane == 0) {
      *rank_out = 0;
      *status_out = 0;
    }
    return;
  }
  {
    const double2 pv = p[i1];
    for (int k = lane; k < d1; k += 32) V[k] = cdiv(p[k], pv);
  }
  fetch(g, rows, cols, n1, n2, !rowfirst, i1, q, lane);
  __syncwarp();
  for (int k = lane; k < d2; k += 32) U[k] = q[k];
  if (lane == 0) {
    list1[0] = i1;
    list2[0] = i2;
    used1[i1] = 1;
    used2[i2] = 1;
  }
  __syncwarp();
  int rk = 1, status = 0;
  double nS = 0.0, prev = 1000.0;
  i2 = warp_argmax(q, used2, d2, lane);
  while (cmag(p[i1]) > eps && cmag(q[i2]) > eps && fabs(prev - nS) >= eps * prev && rk < mn) {
    if (rk >= R) {
      status = 1;
      break;
    }
    __syncwarp();  // every lane has read p[i1] and q[i2] before they are refetched
    fetch(g, rows, cols, n1, n2, rowfirst, i2, p, lane);
    // p[k] -= U[a][i2] V[a][k], a = 0..rk-1 in order (the host's sub_scaled
    // sequence for every element); the coefficients staged in shared memory.
    for (int a = lane; a < rk; a += 32) coef[a] = U[(size_t)a * d2 + i2];
    __syncwarp();
    for (int k = lane; k < d1; k += 32) {
      double2 x = p[k];
#pragma unroll 4
      for (int a = 0; a < rk; ++a) {
        const double2 f = coef[a], w = V[(size_t)a * d1 + k];
        x = make_double2(x.x - (f.x * w.x - f.y * w.y), x.y - (f.x * w.y + f.y * w.x));
      }
      p[k] = x;
    }
    __syncwarp();
    const int n_i1 = warp_argmax(p, used1, d1, lane);
    double2* Vr = V + (size_t)rk * d1;
    {
      const double2 pv = p[n_i1];
      for (int k = lane; k < d1; k += 32) Vr[k] = cdiv(p[k], pv);
    }
    fetch(g, rows, cols, n1, n2, !rowfirst, n_i1, q, lane);
    for (int a = lane; a < rk; a += 32) coef[a] = V[(size_t)a * d1 + n_i1];
    __syncwarp();
    double2* __restrict__ Ur = U + (size_t)rk * d2;
    for (int k = lane; k < d2; k += 32) {
      double2 x = q[k];
#pragma unroll 4
      for (int a = 0; a < rk; ++a) {
        const double2 f = coef[a], w = U[(size_t)a * d2 + k];
        x = make_double2(x.x - (f.x * w.x - f.y * w.y), x.y - (f.x * w.y + f.y * w.x));
      }
      q[k] = x;
      Ur[k] = x;
    }
    __syncwarp();
    const double nu = warp_norm(Ur, d2, lane), nv = warp_norm(Vr, d1, lane);
    if (nu < 1e-8 || nv < 1e-8) break;
    i1 = n_i1;
    if (lane == 0) {
      list1[rk] = i1;
      list2[rk] = i2;
      used1[i1] = 1;
      used2[i2] = 1;
    }
    ++rk;
    if (rk != 2) prev = nS;
    nS = nS * nS + (nu * nv) * (nu * nv);
    for (int a = 0; a < rk; ++a) {
      const double2 cu = warp_cdot(U + (size_t)a * d2, Ur, d2, lane);
      const double2 cv = warp_cdot(V + (size_t)a * d1, Vr, d1, lane);
      const double2 pr = make_double2(cu.x * cv.x - cu.y * cv.y, cu.x * cv.y + cu.y * cv.x);
      nS += 2 * hypot(pr.x, pr.y);
    }
    nS = sqrt(nS);
    __syncwarp();
    i2 = warp_argmax(q, used2, d2, lane);
  }
  if (lane == 0) {
    *rank_out = rk;
    *status_out = status;
  }
}

__global__ void __launch_bounds__(kNcaWarpsPerBlock * 32) nca_kernel(NcaGeomDev g, const NcaTask* __restrict__ tasks,
                                                                    int ntasks, const int* __restrict__ idx, double eps,
                                                                    int* next, int* piv, int* ranks, int* status,
                                                                    double2* scratch, long long warp_scr,
                                                                    unsigned char* flags, long long warp_flags) {
  __shared__ double2 coef_all[kNcaWarpsPerBlock][kNcaRankCapG];
  const int lane = threadIdx.x & 31;
  double2* coef = coef_all[threadIdx.x >> 5];
  const long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  double2* scr = scratch + w * warp_scr;
  unsigned char* used = flags + w * warp_flags;
  for (int iter = 0; iter <= ntasks; ++iter) {
    int t = 0;
    if (lane == 0) t = atomicAdd(next, 1);
    t = __shfl_sync(kFull, t, 0);
    if (t >= ntasks) break;
    aca_task(g, tasks[t], idx, eps, scr, used, piv, ranks + t, status + t, coef, lane);
    __syncwarp();
  }
}

template <class T>
bool upload(T** d, const std::vector<T>& h) {
  *d = nullptr;
  if (h.empty()) return true;
  return cudaMalloc(d, sizeof(T) * h.size()) == cudaSuccess &&
         cudaMemcpy(*d, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice) == cudaSuccess;
}

}  // namespace

struct GpuFar {
  int device = -1;
  NcaGeomDev g{};
  double2* S = nullptr;
  int *xid = nullptr, *yid = nullptr, *xrow = nullptr, *yrow = nullptr, *lcol = nullptr, *lrow = nullptr;
  double* kq = nullptr;
  double seconds_table = 0.0;
  ~GpuFar() {
    cudaFree(S);
    cudaFree(xid);
    cudaFree(yid);
    cudaFree(xrow);
    cudaFree(yrow);
    cudaFree(lcol);
    cudaFree(lrow);
    cudaFree(kq);
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
  const size_t sbytes = sizeof(double2) * (size_t)nkeys * t.rank;
  double *dux = nullptr, *duy = nullptr;
  double2* dM = nullptr;
  std::vector<double2> Mh(t.M.size());
  for (size_t i = 0; i < Mh.size(); ++i) Mh[i] = make_double2(t.M[i].real(), t.M[i].imag());
  const size_t smem = sizeof(double2) * ((size_t)t.rank * kTerms + (size_t)kTableKeys * kTerms);
  bool ok = upload(&dux, t.ux) && upload(&duy, t.uy) && upload(&dM, Mh) && cudaMalloc(&f->S, sbytes) == cudaSuccess &&
            cudaFuncSetAttribute(far_table_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) ==
                cudaSuccess;
  if (ok) {
    const long long blocks = (nkeys + kTableKeys - 1) / kTableKeys;
    far_table_kernel<<<(unsigned)blocks, kTableKeys, smem>>>(dux, duy, (int)ny, nkeys, t.kappa, dM, t.rank, f->S);
    ok = cudaGetLastError() == cudaSuccess && cudaDeviceSynchronize() == cudaSuccess;
  }
  if (ok) {
    static_assert(sizeof(cd) == sizeof(double2), "complex layout");
    ok = cudaMemcpy(S_host, f->S, sbytes, cudaMemcpyDeviceToHost) == cudaSuccess;
  }
  ok = ok && upload(&f->xid, t.xid) && upload(&f->yid, t.yid) && upload(&f->xrow, t.xrow) &&
       upload(&f->yrow, t.yrow) && upload(&f->lcol, t.lcol) && upload(&f->lrow, t.lrow) && upload(&f->kq, t.kq);
  cudaFree(dux);
  cudaFree(duy);
  cudaFree(dM);
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
  const int nt = (int)tasks.size();
  long long warp_scr = 0, warp_flags = 0, npiv = 0;
  for (const NcaTask& t : tasks) {
    if (t.R < 1 || t.R > kNcaRankCapG) return false;
    const long long d = (long long)t.n1 + t.n2;
    warp_scr = std::max(warp_scr, (long long)t.R * d + d);
    warp_flags = std::max(warp_flags, d);
    npiv = std::max(npiv, (long long)t.out_off + 2LL * t.R);
  }
  warp_flags = (warp_flags + 15) / 16 * 16;
  // Warps: one per task up to the GPU's resident warps and an 8 GB scratch.
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, f->device);
  long long warps = std::min<long long>(nt, (long long)std::max(sms, 1) * 48);
  const long long budget = 8LL << 30;
  warps = std::max(1LL, std::min(warps, budget / std::max(1LL, warp_scr * (long long)sizeof(double2))));
  warps = (warps + kNcaWarpsPerBlock - 1) / kNcaWarpsPerBlock * kNcaWarpsPerBlock;
  NcaTask* dt = nullptr;
  int *didx = nullptr, *dnext = nullptr, *dpiv = nullptr, *drank = nullptr, *dstat = nullptr;
  double2* dscr = nullptr;
  unsigned char* dflags = nullptr;
  bool ok = upload(&dt, tasks) && upload(&didx, idx) && cudaMalloc(&dnext, sizeof(int)) == cudaSuccess &&
            cudaMemset(dnext, 0, sizeof(int)) == cudaSuccess &&
            cudaMalloc(&dpiv, sizeof(int) * (size_t)std::max(1LL, npiv)) == cudaSuccess &&
            cudaMalloc(&drank, sizeof(int) * (size_t)nt) == cudaSuccess &&
            cudaMalloc(&dstat, sizeof(int) * (size_t)nt) == cudaSuccess &&
            cudaMalloc(&dscr, sizeof(double2) * (size_t)(warps * warp_scr)) == cudaSuccess &&
            cudaMalloc(&dflags, (size_t)(warps * warp_flags)) == cudaSuccess;
  if (ok) {
    nca_kernel<<<(unsigned)(warps / kNcaWarpsPerBlock), kNcaWarpsPerBlock * 32>>>(
        f->g, dt, nt, didx, eps, dnext, dpiv, drank, dstat, dscr, warp_scr, dflags, warp_flags);
    ok = cudaGetLastError() == cudaSuccess && cudaDeviceSynchronize() == cudaSuccess;
  }
  if (ok) {
    ranks.resize(nt);
    status.resize(nt);
    piv.resize((size_t)std::max(1LL, npiv));
    ok = cudaMemcpy(ranks.data(), drank, sizeof(int) * nt, cudaMemcpyDeviceToHost) == cudaSuccess &&
         cudaMemcpy(status.data(), dstat, sizeof(int) * nt, cudaMemcpyDeviceToHost) == cudaSuccess &&
         cudaMemcpy(piv.data(), dpiv, sizeof(int) * piv.size(), cudaMemcpyDeviceToHost) == cudaSuccess;
  }
  cudaFree(dt);
  cudaFree(didx);
  cudaFree(dnext);
  cudaFree(dpiv);
  cudaFree(drank);
  cudaFree(dstat);
  cudaFree(dscr);
  cudaFree(dflags);
  cudaGetLastError();
  return ok;
}

void gpu_far_close(GpuFar* f) { delete f; }

}  // namespace lsg
