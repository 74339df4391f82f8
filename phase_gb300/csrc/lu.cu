// Direct sparse solve on the device: the drop-in for Phase's
// EigenSparseMatrixSolver (src/Math/EigenSparseMatrixSolver.cpp:5-64), whose
// solve() runs SparseLU::compute (a fresh factorisation) and SparseLU::solve
// on every call, with nIters() = 1 and error() = 0
// (EigenSparseMatrixSolver.h:43-45).
//
// Method: multifrontal LU (Duff & Reid 1983) over a nested-dissection tree
// (lu_host.cpp), FP64 throughout.  Fronts are processed by height (leaves
// first); every front of one height is independent of the others, so one
// launch covers them all:
//
//  * small fronts (order <= kLuSmallM): one CTA assembles the front in
//    shared memory (children's contribution blocks added in child order,
//    then the matrix entries it owns), factorises its k fully summed columns
//    with partial pivoting over its fully summed rows, and writes it back;
//  * large fronts: a warp per row assembles the row in global memory (the
//    same sums in the same order), a CTA adds the owned matrix entries, then
//    kLuPanel-column panels as LAPACK's blocked dgetrf does them: the tall panel
//    is factorised by one CTA with partial pivoting over the front's fully
//    summed rows, its interchanges are applied to the columns right of it
//    and U12 = L11^-1 A12 by TRSM tiles, and the trailing block F22 -= L21
//    U12 by 64 x 64 update tiles.
//
// Row interchanges: inside a panel whole panel rows are exchanged (LAPACK's
// convention), across panels the columns left of the panel are not
// touched (LINPACK's, dgefa/dgesl), so the forward solve applies each
// panel's interchanges to the right-hand side just before that panel's
// eliminations; a small front is one panel per column.  A pivot
// whose magnitude is at most 1e-13 of the largest entry of its column in A
// is replaced by that entry's magnitude and counted: a consistent singular
// system (pure Neumann pressure) then gets one of its solutions instead of
// overflowing.  Nothing is summed atomically except the column maxima
// (order-free), so factorisations and solves repeat bit for bit.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <mutex>

#include "internal.h"
#include "lu.h"

using namespace pg;

namespace {

constexpr int kSmallThreads = 256;
constexpr int kSolveThreads = 512;
constexpr double kPivotRel = 1e-13;

struct LuArgs {
  const LuFront *fronts;
  const int32_t *children, *fidx, *rel, *inv, *e_pos, *e_ptr, *e_src;
  double *pool;
  int32_t *ipiv;                  // per new index: partner row (front-local)
  const unsigned long long *cmax; // per new column: bits of max |a|
  int *n_replaced;
};

__device__ __forceinline__ double col_scale(const LuArgs &a, int col) {
  return __longlong_as_double((long long)a.cmax[col]);
}

// magnitude of the largest entry per column of A (new numbering); the bit
// patterns of non-negative doubles order as the values do
__global__ void k_lu_colmax(int64_t n_src, const int32_t *__restrict__ src_col,
                            const double *__restrict__ vals,
                            unsigned long long *cmax) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= n_src) return;
  const int32_t c = src_col[k];
  if (c < 0) return;
  atomicMax(cmax + c, (unsigned long long)__double_as_longlong(fabs(vals[k])));
}

__device__ __forceinline__ double entry_sum(const LuArgs &a, const double *vals,
                                            int e) {
  double v = 0.;
  for (int q = a.e_ptr[e]; q < a.e_ptr[e + 1]; ++q) v += vals[a.e_src[q]];
  return v;
}

// pivot value with the vanishing-pivot replacement (cs: the column's
// largest magnitude in A)
__device__ __forceinline__ double checked_pivot_scaled(const LuArgs &a,
                                                       double p, double cs) {
  if (fabs(p) <= kPivotRel * cs || p == 0.) {
    atomicAdd(a.n_replaced, 1);
    return cs > 0. ? cs : 1.;
  }
  return p;
}

__device__ __forceinline__ double checked_pivot(const LuArgs &a, double p,
                                                int col) {
  return checked_pivot_scaled(a, p, col_scale(a, col));
}

// ---------------------------------------------------------- small fronts
// T = double for the direct solver; T = float for the dense inverse built
// from it (the two-level preconditioner's coarse matrix, whose inverse is
// applied in FP32), where fpool is the FP32 factor pool.
template <class T>
__global__ void __launch_bounds__(kSmallThreads)
k_lu_small(const int32_t *__restrict__ list, LuArgs a,
           const double *__restrict__ vals, T *__restrict__ fpool) {
  extern __shared__ __align__(16) unsigned char sm_raw[];
  T *F = reinterpret_cast<T *>(sm_raw);
  __shared__ int piv_row;
  __shared__ T piv_inv;
  __shared__ double cscale[kLuSmallM];
  const int tid = threadIdx.x;
  const LuFront f = a.fronts[list[blockIdx.x]];
  const int m = f.m, k = f.k;
  for (int e = tid; e < m * m; e += kSmallThreads) F[e] = T(0);
  for (int c = tid; c < k; c += kSmallThreads) cscale[c] = col_scale(a, f.s0 + c);
  __syncthreads();
  for (int c = 0; c < f.n_child; ++c) {
    const LuFront ch = a.fronts[a.children[f.child_ptr + c]];
    const int u = ch.m - ch.k;
    const T *cb = fpool + ch.off;
    const int32_t *rel = a.rel + ch.rel_off;
    // a warp per contribution row, lanes along it
    for (int ra = tid >> 5; ra < u; ra += kSmallThreads / 32) {
      const int pr = rel[ra] * m;
      const T *src = cb + (size_t)(ch.k + ra) * ch.m + ch.k;
      for (int rb = tid & 31; rb < u; rb += 32) F[pr + rel[rb]] += src[rb];
    }
    __syncthreads();
  }
  for (int e = f.ent_ptr + tid; e < f.ent_end; e += kSmallThreads)
    F[a.e_pos[e]] += (T)entry_sum(a, vals, e);
  __syncthreads();
  for (int c = 0; c < k; ++c) {
    if (tid < 32) {
      double best = -1.;
      int br = c;
      for (int r = c + tid; r < k; r += 32) {
        const double v = fabs((double)F[r * m + c]);
        if (v > best) {
          best = v;
          br = r;
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const double ob = __shfl_down_sync(0xffffffffu, best, o);
        const int orr = __shfl_down_sync(0xffffffffu, br, o);
        if (ob > best || (ob == best && orr < br)) {
          best = ob;
          br = orr;
        }
      }
      if (tid == 0) {
        piv_row = br;
        a.ipiv[f.s0 + c] = br;
        // the exchange of rows c and br (columns c ..) and the pivot
        T p = F[br * m + c];
        if (br != c) {
          for (int j = c; j < m; ++j) {
            const T t = F[c * m + j];
            F[c * m + j] = F[br * m + j];
            F[br * m + j] = t;
          }
        }
        p = (T)checked_pivot_scaled(a, (double)p, cscale[c]);
        F[c * m + c] = p;
        piv_inv = T(1) / p;  // one division per pivot
      }
    }
    __syncthreads();
    const T rp = piv_inv;
    // multipliers and the rank-1 update: a warp per row, lanes along it
    for (int i = c + 1 + (tid >> 5); i < m; i += kSmallThreads / 32) {
      const T l = F[i * m + c] * rp;
      for (int j = c + 1 + (tid & 31); j < m; j += 32)
        F[i * m + j] -= l * F[c * m + j];
      __syncwarp();
      if ((tid & 31) == 0) F[i * m + c] = l;
    }
    __syncthreads();
  }
  T *out = fpool + f.off;
  for (int e = tid; e < m * m; e += kSmallThreads) out[e] = F[e];
}

// ---------------------------------------------------------- large fronts
// one warp per (front, row): children's contribution rows, in child order
__global__ void __launch_bounds__(256)
k_lu_assemble_rows(int n_tasks, const int32_t *__restrict__ rows, LuArgs a) {
  const int task = blockIdx.x * 8 + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (task >= n_tasks) return;
  const int t = rows[2 * task], i = rows[2 * task + 1];
  const LuFront f = a.fronts[t];
  const int m = f.m;
  double *row = a.pool + f.off + (size_t)i * m;
  for (int j = lane; j < m; j += 32) {
    double v = 0.;
    for (int c = 0; c < f.n_child; ++c) {
      const LuFront ch = a.fronts[a.children[f.child_ptr + c]];
      const int32_t *inv = a.inv + ch.inv_off;
      const int ai = inv[i];
      if (ai < 0) continue;
      const int bj = inv[j];
      if (bj >= 0)
        v += a.pool[ch.off + (size_t)(ch.k + ai) * ch.m + ch.k + bj];
    }
    row[j] = v;
  }
}

__global__ void __launch_bounds__(256)
k_lu_scatter(const int32_t *__restrict__ list, LuArgs a,
             const double *__restrict__ vals) {
  const LuFront f = a.fronts[list[blockIdx.x]];
  double *F = a.pool + f.off;
  for (int e = f.ent_ptr + threadIdx.x; e < f.ent_end; e += 256)
    F[a.e_pos[e]] += entry_sum(a, vals, e);
}

// panel q of the large fronts, one CTA per front: the tall panel (rows
// c0 .. m-1, columns c0 .. c0+b-1) is factorised with partial pivoting over
// the fully summed rows c .. k-1 of each column c; an interchange swaps the
// whole panel rows (LAPACK's convention inside a panel), which the TRSM
// kernel then applies to the columns right of it.  Warps own rows, lanes
// the panel's columns; a warp keeps kPanelBatch rows' loads in flight, and
// the candidates for the next column's pivot are ranked as the rows are
// updated, so each step reads the panel once.
constexpr int kPanelThreads = 1024;
constexpr int kPanelBatch = 4;

__device__ __forceinline__ void better(double &best, int &br, double v, int r) {
  if (v > best || (v == best && r < br)) {
    best = v;
    br = r;
  }
}

__global__ void __launch_bounds__(kPanelThreads)
k_lu_panel(const int32_t *__restrict__ list, int q, LuArgs a) {
  constexpr int NW = kPanelThreads / 32;
  __shared__ double wbest[NW];
  __shared__ int wrow[NW];
  __shared__ double piv_inv;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const LuFront f = a.fronts[list[blockIdx.x]];
  const int m = f.m, k = f.k, c0 = q * kLuPanel, b = min(kLuPanel, k - c0);
  double *F = a.pool + f.off;
  // candidates for the first column: a thread per row
  double best = -1.;
  int br = c0;
  for (int r = c0 + tid; r < k; r += kPanelThreads)
    better(best, br, fabs(F[(size_t)r * m + c0]), r);
  for (int s = 0; s < b; ++s) {
    const int c = c0 + s;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double ob = __shfl_down_sync(0xffffffffu, best, o);
      const int orr = __shfl_down_sync(0xffffffffu, br, o);
      better(best, br, ob, orr);
    }
    if (lane == 0) {
      wbest[warp] = best;
      wrow[warp] = br;
    }
    __syncthreads();
    if (warp == 0) {
      best = wbest[lane];
      br = wrow[lane];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const double ob = __shfl_down_sync(0xffffffffu, best, o);
        const int orr = __shfl_down_sync(0xffffffffu, br, o);
        better(best, br, ob, orr);
      }
      const int r = __shfl_sync(0xffffffffu, br, 0);
      if (r != c && lane < b) {
        const double t = F[(size_t)c * m + c0 + lane];
        F[(size_t)c * m + c0 + lane] = F[(size_t)r * m + c0 + lane];
        F[(size_t)r * m + c0 + lane] = t;
      }
      __syncwarp();
      if (lane == 0) {
        a.ipiv[f.s0 + c] = r;
        const double p = checked_pivot(a, F[(size_t)c * m + c], f.s0 + c);
        F[(size_t)c * m + c] = p;
        piv_inv = 1. / p;  // one division per pivot
      }
    }
    __syncthreads();
    const double rp = piv_inv;
    const double prow = lane < b ? F[(size_t)c * m + c0 + lane] : 0.;
    best = -1.;
    br = c + 1;
    for (int i0 = c + 1 + warp; i0 < m; i0 += NW * kPanelBatch) {
      double v[kPanelBatch];
#pragma unroll
      for (int u = 0; u < kPanelBatch; ++u) {
        const int i = i0 + u * NW;
        v[u] = i < m && lane < b ? F[(size_t)i * m + c0 + lane] : 0.;
      }
#pragma unroll
      for (int u = 0; u < kPanelBatch; ++u) {
        const int i = i0 + u * NW;
        const double l = __shfl_sync(0xffffffffu, v[u], s) * rp;
        if (lane == s) v[u] = l;
        else if (lane > s) v[u] -= l * prow;
        if (i < m && lane >= s && lane < b) F[(size_t)i * m + c0 + lane] = v[u];
        // the next column's candidate of this row (fully summed rows only;
        // the condition is the same for the whole warp)
        if (s + 1 < b && i < k) {
          const double nv = fabs(__shfl_sync(0xffffffffu, v[u], s + 1));
          better(best, br, nv, i);
        }
      }
    }
    __syncthreads();
  }
}

// U12 tiles of panel q: the panel's interchanges replayed on the columns
// right of it (rows c0 .. k-1, in global memory), then U12 = L11^-1 A12
// (a thread per column)
__global__ void __launch_bounds__(kLuTrsmCols)
k_lu_trsm(const int32_t *__restrict__ tasks, int q, LuArgs a) {
  __shared__ double D[kLuPanel][kLuPanel + 1];
  __shared__ int pr[kLuPanel];
  const int tid = threadIdx.x;
  const int t = tasks[3 * blockIdx.x], t0 = tasks[3 * blockIdx.x + 2];
  const LuFront f = a.fronts[t];
  const int m = f.m, c0 = q * kLuPanel, b = min(kLuPanel, f.k - c0);
  double *F = a.pool + f.off;
  for (int e = tid; e < kLuPanel * kLuPanel; e += kLuTrsmCols) {
    const int r = e / kLuPanel, c = e % kLuPanel;
    D[r][c] = r < b && c < b ? F[(size_t)(c0 + r) * m + c0 + c] : 0.;
  }
  if (tid < kLuPanel) pr[tid] = tid < b ? a.ipiv[f.s0 + c0 + tid] : 0;
  __syncthreads();
  const int j = c0 + b + t0 + tid;
  if (j >= m) return;
  for (int s = 0; s < b; ++s) {
    const int r = pr[s];
    if (r != c0 + s) {
      const double x = F[(size_t)(c0 + s) * m + j];
      F[(size_t)(c0 + s) * m + j] = F[(size_t)r * m + j];
      F[(size_t)r * m + j] = x;
    }
  }
  double T[kLuPanel];
#pragma unroll
  for (int r = 0; r < kLuPanel; ++r) T[r] = r < b ? F[(size_t)(c0 + r) * m + j] : 0.;
#pragma unroll
  for (int s = 0; s < kLuPanel; ++s) {
#pragma unroll
    for (int i = s + 1; i < kLuPanel; ++i) T[i] -= D[i][s] * T[s];
  }
#pragma unroll
  for (int r = 0; r < kLuPanel; ++r)
    if (r < b) F[(size_t)(c0 + r) * m + j] = T[r];
}

// trailing update of panel q: F22 -= L21 U12 on a 64 x 64 tile; each thread
// keeps 4 x 4 sums, accumulated over the panel's pivots in order
__global__ void __launch_bounds__(256)
k_lu_update(const int32_t *__restrict__ tasks, int q, LuArgs a) {
  __shared__ double Ls[kLuUpd][kLuPanel + 1];
  __shared__ double Us[kLuPanel][kLuUpd + 1];
  const int tid = threadIdx.x;
  const int t = tasks[3 * blockIdx.x], i0 = tasks[3 * blockIdx.x + 1],
            j0 = tasks[3 * blockIdx.x + 2];
  const LuFront f = a.fronts[t];
  const int m = f.m, c0 = q * kLuPanel, b = min(kLuPanel, f.k - c0);
  const int base = c0 + b;
  double *F = a.pool + f.off;
  for (int e = tid; e < kLuUpd * kLuPanel; e += 256) {
    const int r = e / kLuPanel, s = e % kLuPanel;
    const int i = base + i0 + r;
    Ls[r][s] = i < m && s < b ? F[(size_t)i * m + c0 + s] : 0.;
  }
  for (int e = tid; e < kLuPanel * kLuUpd; e += 256) {
    const int s = e / kLuUpd, c = e % kLuUpd;
    const int j = base + j0 + c;
    Us[s][c] = j < m && s < b ? F[(size_t)(c0 + s) * m + j] : 0.;
  }
  __syncthreads();
  const int tx = tid & 15, ty = tid >> 4;
  double acc[4][4] = {};
  for (int s = 0; s < b; ++s) {
    double lv[4], uv[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) lv[r] = Ls[ty * 4 + r][s];
#pragma unroll
    for (int c = 0; c < 4; ++c) uv[c] = Us[s][tx * 4 + c];
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int c = 0; c < 4; ++c) acc[r][c] += lv[r] * uv[c];
  }
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int i = base + i0 + ty * 4 + r;
    if (i >= m) continue;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const int j = base + j0 + tx * 4 + c;
      if (j < m) F[(size_t)i * m + j] -= acc[r][c];
    }
  }
}

// ---------------------------------------------------------------- solves
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// out[i] -= F[i][c0 .. c0+b) . vec for the rows i = first, first + 16, ...
// below last: a warp per row (lanes along the block, lane l holding vec's
// entry l), four rows' loads in flight
__device__ __forceinline__ void gemv_rows(const double *F, int m, int c0, int b,
                                          int lane, double vl, int first,
                                          int last, double *out) {
  constexpr int NW = kSolveThreads / 32, R = 4;
  for (int i0 = first; i0 < last; i0 += NW * R) {
    double part[R];
#pragma unroll
    for (int u = 0; u < R; ++u) {
      const int i = i0 + u * NW;
      part[u] = i < last && lane < b ? F[(size_t)i * m + c0 + lane] * vl : 0.;
    }
#pragma unroll
    for (int u = 0; u < R; ++u) {
      const double sum = warp_sum(part[u]);
      const int i = i0 + u * NW;
      if (lane == 0 && i < last) out[i] -= sum;
    }
  }
}

// forward elimination of one height: b (new numbering) -> y for the fully
// summed rows, contribution vectors for the update rows
__global__ void __launch_bounds__(kSolveThreads)
k_lu_fwd(const int32_t *__restrict__ list, LuArgs a,
         const double *__restrict__ bn, double *__restrict__ y,
         double *__restrict__ cpool) {
  extern __shared__ double w[];
  __shared__ double D[kLuPanel][kLuPanel + 1];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int ft = list[blockIdx.x];
  const LuFront f = a.fronts[ft];
  const int m = f.m, k = f.k;
  const double *F = a.pool + f.off;
  for (int i = tid; i < m; i += kSolveThreads) w[i] = i < k ? bn[f.s0 + i] : 0.;
  __syncthreads();
  for (int c = 0; c < f.n_child; ++c) {
    const LuFront ch = a.fronts[a.children[f.child_ptr + c]];
    const int u = ch.m - ch.k;
    const int32_t *rel = a.rel + ch.rel_off;
    const double *cv = cpool + ch.coff;
    for (int e = tid; e < u; e += kSolveThreads) w[rel[e]] += cv[e];
    __syncthreads();
  }
  if (!f.large) {
    for (int c = 0; c < k; ++c) {
      if (tid == 0) {
        const int r = a.ipiv[f.s0 + c];
        if (r != c) {
          const double x = w[c];
          w[c] = w[r];
          w[r] = x;
        }
      }
      __syncthreads();
      const double wc = w[c];
      for (int i = c + 1 + tid; i < m; i += kSolveThreads)
        w[i] -= F[(size_t)i * m + c] * wc;
      __syncthreads();
    }
  } else {
    for (int c0 = 0; c0 < k; c0 += kLuPanel) {
      const int b = min(kLuPanel, k - c0);
      for (int e = tid; e < kLuPanel * kLuPanel; e += kSolveThreads) {
        const int r = e / kLuPanel, c = e % kLuPanel;
        D[r][c] = r < b && c < b ? F[(size_t)(c0 + r) * m + c0 + c] : 0.;
      }
      __syncthreads();
      if (warp == 0) {
        // the panel's interchanges (rows c0 .. k-1), then L11
        if (lane == 0)
          for (int s = 0; s < b; ++s) {
            const int r = a.ipiv[f.s0 + c0 + s];
            if (r != c0 + s) {
              const double x = w[c0 + s];
              w[c0 + s] = w[r];
              w[r] = x;
            }
          }
        __syncwarp();
        for (int s = 0; s < b; ++s) {
          const double ws = w[c0 + s];
          if (lane > s && lane < b) w[c0 + lane] -= D[lane][s] * ws;
          __syncwarp();
        }
      }
      __syncthreads();
      const double wl = lane < b ? w[c0 + lane] : 0.;
      gemv_rows(F, m, c0, b, lane, wl, c0 + b + warp, m, w);
      __syncthreads();
    }
  }
  for (int i = tid; i < m; i += kSolveThreads) {
    if (i < k) y[f.s0 + i] = w[i];
    else cpool[f.coff + i - k] = w[i];
  }
}

// back substitution of one height: x of the fully summed variables from y
// and the x of the update variables (solved by the ancestors)
__global__ void __launch_bounds__(kSolveThreads)
k_lu_bwd(const int32_t *__restrict__ list, LuArgs a,
         const double *__restrict__ y, double *__restrict__ xn) {
  extern __shared__ double sm[];
  __shared__ double D[kLuPanel][kLuPanel + 1];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const LuFront f = a.fronts[list[blockIdx.x]];
  const int m = f.m, k = f.k, u = m - k;
  double *r = sm, *xu = sm + k;
  const double *F = a.pool + f.off;
  for (int i = tid; i < m; i += kSolveThreads) {
    if (i < k) r[i] = y[f.s0 + i];
    else xu[i - k] = xn[a.fidx[f.idx + i]];
  }
  __syncthreads();
  if (u > 0)
    for (int i = warp; i < k; i += kSolveThreads / 32) {
      double part = 0.;
      for (int j = lane; j < u; j += 32) part += F[(size_t)i * m + k + j] * xu[j];
      const double sum = warp_sum(part);
      if (lane == 0) r[i] -= sum;
    }
  __syncthreads();
  if (!f.large) {
    for (int c = k - 1; c >= 0; --c) {
      if (tid == 0) r[c] /= F[(size_t)c * m + c];
      __syncthreads();
      const double xc = r[c];
      for (int i = tid; i < c; i += kSolveThreads) r[i] -= F[(size_t)i * m + c] * xc;
      __syncthreads();
    }
  } else {
    const int nb = (k + kLuPanel - 1) / kLuPanel;
    for (int qb = nb - 1; qb >= 0; --qb) {
      const int c0 = qb * kLuPanel, b = min(kLuPanel, k - c0);
      for (int e = tid; e < kLuPanel * kLuPanel; e += kSolveThreads) {
        const int rr = e / kLuPanel, c = e % kLuPanel;
        D[rr][c] = rr < b && c < b ? F[(size_t)(c0 + rr) * m + c0 + c] : 0.;
      }
      __syncthreads();
      if (warp == 0) {
        for (int s = b - 1; s >= 0; --s) {
          if (lane == 0) r[c0 + s] /= D[s][s];
          __syncwarp();
          const double xs = r[c0 + s];
          if (lane < s) r[c0 + lane] -= D[lane][s] * xs;
          __syncwarp();
        }
      }
      __syncthreads();
      const double xl = lane < b ? r[c0 + lane] : 0.;
      gemv_rows(F, m, c0, b, lane, xl, warp, c0, r);
      __syncthreads();
    }
  }
  for (int i = tid; i < k; i += kSolveThreads) xn[f.s0 + i] = r[i];
}

__global__ void k_lu_gather(int n, const int32_t *__restrict__ perm,
                            const double *__restrict__ src, double scale,
                            double *__restrict__ dst) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = scale * src[perm[i]];
}

__global__ void k_lu_scale(int n, const double *__restrict__ src, double scale,
                           double *__restrict__ dst) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = scale * src[i];
}

__global__ void k_lu_scatter_x(int n, const int32_t *__restrict__ perm,
                               const double *__restrict__ src,
                               double *__restrict__ dst) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[perm[i]] = src[i];
}

// ||b - A x||^2 and ||b||^2 partial sums per block over the caller's CSR
// (placeholder columns skipped), original numbering
__global__ void __launch_bounds__(256)
k_lu_residual(int n, const int32_t *__restrict__ rp, const int32_t *__restrict__ ci,
              const double *__restrict__ v, const double *__restrict__ x,
              const double *__restrict__ b, double *__restrict__ part) {
  __shared__ double s1[256], s2[256];
  const int i = blockIdx.x * 256 + threadIdx.x;
  double rr = 0., bb = 0.;
  if (i < n) {
    double ax = 0.;
    for (int e = rp[i]; e < rp[i + 1]; ++e) {
      const int c = ci[e];
      if (c >= 0) ax += v[e] * x[c];
    }
    const double r = b[i] - ax;
    rr = r * r;
    bb = b[i] * b[i];
  }
  s1[threadIdx.x] = rr;
  s2[threadIdx.x] = bb;
  __syncthreads();
  for (int h = 128; h > 0; h >>= 1) {
    if (threadIdx.x < h) {
      s1[threadIdx.x] += s1[threadIdx.x + h];
      s2[threadIdx.x] += s2[threadIdx.x + h];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = s1[0];
    part[2 * blockIdx.x + 1] = s2[0];
  }
}

// ------------------------------------------------- dense inverse (FP32)
// A^-1 column tile by column tile: the identity (new numbering) as
// kInvCols right-hand sides per CTA, forward eliminated front by front (LINPACK
// order, FP64 factors read and rounded to FP32), then back substituted
// from the root down; a front's tile whose columns lie outside its subtree
// is zero and is only written as zeros.  Small fronts only (m <= kLuSmallM).
constexpr int kInvCols = 128;  // right-hand-side columns per CTA

// Each thread owns one column of the right-hand sides (W[i][thread], a
// column per shared-memory bank) and runs the whole elimination of its
// column; the front's factor is staged once in shared memory and only
// broadcast-read, so no barrier is needed inside the loops.
__global__ void __launch_bounds__(kInvCols)
k_lu_inv_fwd(const int32_t *__restrict__ list, LuArgs a,
             const float *__restrict__ pool32, int n, float *__restrict__ Y,
             float *__restrict__ CP) {
  extern __shared__ float smf[];
  const int cc = threadIdx.x;
  const LuFront f = a.fronts[list[blockIdx.x]];
  const int m = f.m, k = f.k, j0 = blockIdx.y * kInvCols;
  const int j = j0 + cc;
  float *Fs = smf, *W = smf + m * m;  // W[i * kInvCols + cc]
  const bool live = j0 + kInvCols > f.first && j0 < f.s0 + k;
  if (live) {
    const float *F32 = pool32 + f.off;
    for (int e = cc; e < m * m; e += kInvCols) Fs[e] = F32[e];
  }
  for (int i = 0; i < m; ++i)
    W[i * kInvCols + cc] = live && i < k && f.s0 + i == j ? 1.f : 0.f;
  __syncthreads();
  if (live && j < n) {
    for (int c = 0; c < f.n_child; ++c) {
      const LuFront ch = a.fronts[a.children[f.child_ptr + c]];
      const int u = ch.m - ch.k;
      const int32_t *rel = a.rel + ch.rel_off;
      // eight independent loads in flight per batch
      for (int e0 = 0; e0 < u; e0 += 8) {
        float v[8];
#pragma unroll
        for (int q = 0; q < 8; ++q)
          v[q] = e0 + q < u ? CP[(size_t)(ch.coff + e0 + q) * n + j] : 0.f;
#pragma unroll
        for (int q = 0; q < 8; ++q)
          if (e0 + q < u) W[rel[e0 + q] * kInvCols + cc] += v[q];
      }
    }
    for (int c = 0; c < k; ++c) {
      const int r = a.ipiv[f.s0 + c];
      float wc = W[c * kInvCols + cc];
      if (r != c) {
        const float x = W[r * kInvCols + cc];
        W[r * kInvCols + cc] = wc;
        W[c * kInvCols + cc] = x;
        wc = x;
      }
      for (int i = c + 1; i < m; ++i) W[i * kInvCols + cc] -= Fs[i * m + c] * wc;
    }
  }
  if (j >= n) return;
  for (int i = 0; i < m; ++i) {
    if (i < k) Y[(size_t)(f.s0 + i) * n + j] = W[i * kInvCols + cc];
    else CP[(size_t)(f.coff + i - k) * n + j] = W[i * kInvCols + cc];
  }
}

__global__ void __launch_bounds__(kInvCols)
k_lu_inv_bwd(const int32_t *__restrict__ list, LuArgs a,
             const float *__restrict__ pool32, int n, float *__restrict__ Y) {
  extern __shared__ float smf[];
  const int cc = threadIdx.x;
  const LuFront f = a.fronts[list[blockIdx.x]];
  const int m = f.m, k = f.k, j = blockIdx.y * kInvCols + cc;
  float *Fs = smf, *W = smf + m * m;
  {
    const float *F32 = pool32 + f.off;
    for (int e = cc; e < m * m; e += kInvCols) Fs[e] = F32[e];
  }
  __syncthreads();
  if (j >= n) return;
  for (int i0 = 0; i0 < m; i0 += 8) {  // eight loads in flight per batch
    float v[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int i = i0 + q;
      v[q] = i >= m ? 0.f
             : i < k ? Y[(size_t)(f.s0 + i) * n + j]
                     : Y[(size_t)a.fidx[f.idx + i] * n + j];
    }
#pragma unroll
    for (int q = 0; q < 8; ++q)
      if (i0 + q < m) W[(i0 + q) * kInvCols + cc] = v[q];
  }
  // r = y_S - U12 x_U, then U11 back substitution
  for (int i = 0; i < k; ++i) {
    float acc = 0.f;
    for (int u = k; u < m; ++u) acc += Fs[i * m + u] * W[u * kInvCols + cc];
    W[i * kInvCols + cc] -= acc;
  }
  for (int c = k - 1; c >= 0; --c) {
    const float xc = W[c * kInvCols + cc] / Fs[c * m + c];
    W[c * kInvCols + cc] = xc;
    for (int i = 0; i < c; ++i) W[i * kInvCols + cc] -= Fs[i * m + c] * xc;
  }
  for (int i = 0; i < k; ++i) Y[(size_t)(f.s0 + i) * n + j] = W[i * kInvCols + cc];
}

// out[I][J] = X[iperm[I]][iperm[J]] (caller's numbering)
__global__ void k_lu_inv_out(int n, const int32_t *__restrict__ iperm,
                             const float *__restrict__ X, float *__restrict__ out) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= (int64_t)n * n) return;
  const int I = (int)(e / n), J = (int)(e % n);
  out[e] = X[(size_t)iperm[I] * n + iperm[J]];
}

int grid_of(int64_t n, int b) { return (int)((n + b - 1) / b); }

// opt in to large dynamic shared memory once per process
int lu_smem_setup() {
  static std::once_flag once;
  static cudaError_t err = cudaSuccess;
  std::call_once(once, [] {
    const int big = 200 * 1024;
    err = cudaFuncSetAttribute(k_lu_small<double>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize, big);
    if (err == cudaSuccess)
      err = cudaFuncSetAttribute(k_lu_small<float>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, big);
    if (err == cudaSuccess)
      err = cudaFuncSetAttribute(k_lu_fwd,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, big);
    if (err == cudaSuccess)
      err = cudaFuncSetAttribute(k_lu_bwd,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  });
  PG_CUDA(err);
  return PG_OK;
}

}  // namespace

struct pg_lu {
  int64_t rank = 0;
  LuSymbolic s;
  bool analysed = false;
  uint64_t eqn_pattern = 0;  // pattern id of the device equation, 0 = CSR
  bool have_vals = false, have_rhs = false, factored = false, solved = false;
  std::vector<double> row_x, row_y;
  std::vector<int32_t> raw_rp, raw_ci;  // host copy of the caller's pattern
  // device symbolic data
  DevBuf<LuFront> fronts;
  DevBuf<int32_t> children, fidx, rel, inv, e_pos, e_ptr, e_src, src_col, perm;
  DevBuf<int32_t> h_small, h_large, h_all, large_rows, pt_diag, pt_trsm, pt_upd;
  // numeric data
  DevBuf<double> pool, cpool, bn, y, xn, x, b, vals_st, rhs_st, part;
  DevBuf<int32_t> ipiv, rp_st, ci_st;
  DevBuf<unsigned long long> cmax;
  DevBuf<int> n_rep;
  // dense inverse (lu_inverse_run): the n x n result in new numbering, the
  // contribution rows of every front x n, the factor pool in FP32, old ->
  // new numbering
  DevBuf<float> inv_y, inv_cp, pool32;
  int inv_launches = 0;
  bool inv_captured = false;
  DevBuf<int32_t> iperm;
  // the CSR the last factorisation read (device), for the residual
  const int32_t *m_rp = nullptr, *m_ci = nullptr;
  const double *m_vals = nullptr;
  int replaced = 0;
  double analyse_ms = 0., factor_ms = 0., solve_ms = 0., rel_residual = -1.;
  cudaEvent_t ev[4] = {};
};

namespace {

LuArgs args_of(pg_lu *L) {
  LuArgs a;
  a.fronts = L->fronts.p;
  a.children = L->children.p;
  a.fidx = L->fidx.p;
  a.rel = L->rel.p;
  a.inv = L->inv.p;
  a.e_pos = L->e_pos.p;
  a.e_ptr = L->e_ptr.p;
  a.e_src = L->e_src.p;
  a.pool = L->pool.p;
  a.ipiv = L->ipiv.p;
  a.cmax = L->cmax.p;
  a.n_replaced = L->n_rep.p;
  return a;
}

int analyse_and_upload(pg_lu *L, const int32_t *rp, const int32_t *ci,
                       const double *x, const double *y, int leaf = 64) {
  auto t0 = std::chrono::steady_clock::now();
  int rc = lu_analyse(L->rank, rp, ci, x, y, leaf, L->s);
  if (rc) return rc;
  const LuSymbolic &s = L->s;
  PG_CHECK_ARG(s.max_m <= 25000, "pg_lu: a front is too large (the matrix "
                                 "is too dense for this solver)");
  rc = lu_smem_setup();
  if (rc) return rc;
  PG_CUDA(L->fronts.upload(s.fronts));
  PG_CUDA(L->children.upload(s.children));
  PG_CUDA(L->fidx.upload(s.fidx));
  PG_CUDA(L->rel.upload(s.rel));
  PG_CUDA(L->inv.upload(s.inv));
  PG_CUDA(L->e_pos.upload(s.e_pos));
  PG_CUDA(L->e_ptr.upload(s.e_ptr));
  PG_CUDA(L->e_src.upload(s.e_src));
  PG_CUDA(L->src_col.upload(s.src_col));
  PG_CUDA(L->perm.upload(s.perm));
  PG_CUDA(L->h_small.upload(s.h_small));
  PG_CUDA(L->h_large.upload(s.h_large));
  PG_CUDA(L->h_all.upload(s.h_all));
  PG_CUDA(L->large_rows.upload(s.large_rows));
  PG_CUDA(L->pt_diag.upload(s.pt_diag));
  PG_CUDA(L->pt_trsm.upload(s.pt_trsm));
  PG_CUDA(L->pt_upd.upload(s.pt_upd));
  PG_CUDA(L->pool.reserve(s.pool));
  PG_CUDA(L->cpool.reserve(s.cpool));
  PG_CUDA(L->ipiv.reserve(s.n));
  PG_CUDA(L->cmax.reserve(s.n));
  PG_CUDA(L->bn.reserve(s.n));
  PG_CUDA(L->y.reserve(s.n));
  PG_CUDA(L->xn.reserve(s.n));
  PG_CUDA(L->x.reserve(s.n));
  PG_CUDA(L->b.reserve(s.n));
  PG_CUDA(L->n_rep.reserve(1));
  PG_CUDA(L->part.reserve(2 * (size_t)grid_of(s.n, 256)));
  L->analyse_ms = std::chrono::duration<double, std::milli>(
                      std::chrono::steady_clock::now() - t0)
                      .count();
  L->analysed = true;
  L->factored = false;
  return PG_OK;
}

// the numeric factorisation of the values vals (caller's index space);
// f32: small fronts only, in FP32 into pool32 (the dense-inverse path)
int factor(pg_lu *L, const double *vals, cudaStream_t st, bool f32 = false) {
  const LuSymbolic &s = L->s;
  LuArgs a = args_of(L);
  PG_CUDA(cudaEventRecord(L->ev[0], st));
  PG_CUDA(cudaMemsetAsync(L->cmax.p, 0, s.n * sizeof(unsigned long long), st));
  PG_CUDA(cudaMemsetAsync(L->n_rep.p, 0, sizeof(int), st));
  if (s.n_src > 0) {
    k_lu_colmax<<<grid_of(s.n_src, 256), 256, 0, st>>>(s.n_src, L->src_col.p,
                                                       vals, L->cmax.p);
    count_launches(1);
  }
  for (int h = 0; h < s.n_heights; ++h) {
    const int ns = s.h_small_ptr[h + 1] - s.h_small_ptr[h];
    if (ns > 0) {
      int mm = 0;
      for (int i = s.h_small_ptr[h]; i < s.h_small_ptr[h + 1]; ++i)
        mm = std::max(mm, s.fronts[s.h_small[i]].m);
      if (f32)
        k_lu_small<float><<<ns, kSmallThreads, (size_t)mm * mm * sizeof(float),
                            st>>>(L->h_small.p + s.h_small_ptr[h], a, vals,
                                  L->pool32.p);
      else
        k_lu_small<double><<<ns, kSmallThreads, (size_t)mm * mm * sizeof(double),
                             st>>>(L->h_small.p + s.h_small_ptr[h], a, vals,
                                   L->pool.p);
      count_launches(1);
    }
    const int nl = s.h_large_ptr[h + 1] - s.h_large_ptr[h];
    if (nl == 0) continue;
    const int nr = s.h_rows_ptr[h + 1] - s.h_rows_ptr[h];
    k_lu_assemble_rows<<<grid_of(nr, 8), 256, 0, st>>>(
        nr, L->large_rows.p + 2 * (size_t)s.h_rows_ptr[h], a);
    k_lu_scatter<<<nl, 256, 0, st>>>(L->h_large.p + s.h_large_ptr[h], a, vals);
    count_launches(2);
    for (const LuSymbolic::PanelStep &p : s.steps) {
      if (p.height != h) continue;
      k_lu_panel<<<p.diag_end - p.diag_ptr, kPanelThreads, 0, st>>>(
          L->pt_diag.p + p.diag_ptr, p.panel, a);
      count_launches(1);
      if (p.trsm_end > p.trsm_ptr) {
        k_lu_trsm<<<p.trsm_end - p.trsm_ptr, kLuTrsmCols, 0, st>>>(
            L->pt_trsm.p + 3 * (size_t)p.trsm_ptr, p.panel, a);
        count_launches(1);
      }
      if (p.upd_end > p.upd_ptr) {
        k_lu_update<<<p.upd_end - p.upd_ptr, 256, 0, st>>>(
            L->pt_upd.p + 3 * (size_t)p.upd_ptr, p.panel, a);
        count_launches(1);
      }
    }
  }
  PG_CUDA(cudaGetLastError());
  PG_CUDA(cudaEventRecord(L->ev[1], st));
  L->factored = true;
  return PG_OK;
}

int solve_now(pg_lu *L) {
  cudaStream_t st = stream();
  const LuSymbolic &s = L->s;
  LuArgs a = args_of(L);
  const int n = (int)s.n;
  PG_CUDA(cudaEventRecord(L->ev[2], st));
  k_lu_gather<<<grid_of(n, 256), 256, 0, st>>>(n, L->perm.p, L->b.p, 1.0, L->bn.p);
  count_launches(1);
  for (int h = 0; h < s.n_heights; ++h) {
    const int nf = s.h_all_ptr[h + 1] - s.h_all_ptr[h];
    const size_t smem = (size_t)s.h_maxm[h] * sizeof(double);
    k_lu_fwd<<<nf, kSolveThreads, smem, st>>>(L->h_all.p + s.h_all_ptr[h], a,
                                              L->bn.p, L->y.p, L->cpool.p);
    count_launches(1);
  }
  for (int h = s.n_heights - 1; h >= 0; --h) {
    const int nf = s.h_all_ptr[h + 1] - s.h_all_ptr[h];
    const size_t smem = (size_t)s.h_maxm[h] * sizeof(double);
    k_lu_bwd<<<nf, kSolveThreads, smem, st>>>(L->h_all.p + s.h_all_ptr[h], a,
                                              L->y.p, L->xn.p);
    count_launches(1);
  }
  k_lu_scatter_x<<<grid_of(n, 256), 256, 0, st>>>(n, L->perm.p, L->xn.p, L->x.p);
  count_launches(1);
  const int g = grid_of(n, 256);
  k_lu_residual<<<g, 256, 0, st>>>(n, L->m_rp, L->m_ci, L->m_vals, L->x.p,
                                   L->b.p, L->part.p);
  count_launches(1);
  PG_CUDA(cudaGetLastError());
  PG_CUDA(cudaEventRecord(L->ev[3], st));
  std::vector<double> part(2 * (size_t)g);
  PG_CUDA(cudaMemcpyAsync(part.data(), L->part.p, part.size() * sizeof(double),
                          cudaMemcpyDeviceToHost, st));
  int rep = 0;
  PG_CUDA(cudaMemcpyAsync(&rep, L->n_rep.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  PG_CUDA(cudaStreamSynchronize(st));
  double rr = 0., bb = 0.;
  for (int i = 0; i < g; ++i) {
    rr += part[2 * i];
    bb += part[2 * i + 1];
  }
  L->rel_residual = bb > 0. ? std::sqrt(rr / bb) : std::sqrt(rr);
  L->replaced = rep;
  float ms = 0.f;
  PG_CUDA(cudaEventElapsedTime(&ms, L->ev[2], L->ev[3]));
  L->solve_ms = ms;
  L->solved = true;
  if (!std::isfinite(L->rel_residual)) {
    set_error("pg_lu_solve: non-finite solution");
    return PG_NON_FINITE;
  }
  return PG_OK;
}

}  // namespace

extern "C" int pg_lu_create(pg_lu **out) {
  PG_CHECK_ARG(out, "pg_lu_create: NULL out");
  *out = nullptr;
  int dev_count = 0;
  if (cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count == 0) {
    cudaGetLastError();
    set_error("no CUDA device available: libphase_gb300 has no CPU path");
    return PG_CUDA_ERROR;
  }
  pg_lu *L = new pg_lu();
  for (auto &e : L->ev) {
    if (cudaEventCreate(&e) != cudaSuccess) {
      delete L;
      set_error("pg_lu_create: cudaEventCreate failed");
      return PG_CUDA_ERROR;
    }
  }
  *out = L;
  return PG_OK;
}

extern "C" int pg_lu_destroy(pg_lu *L) {
  if (!L) return PG_OK;
  cudaStreamSynchronize(stream());
  for (auto &e : L->ev)
    if (e) cudaEventDestroy(e);
  delete L;
  return PG_OK;
}

extern "C" int pg_lu_set_rank(pg_lu *L, int64_t n) {
  PG_CHECK_ARG(L && n > 0, "pg_lu_set_rank: bad argument");
  PG_CHECK_ARG(n < ((int64_t)1 << 31), "pg_lu_set_rank: rank too large");
  if (L->rank != n) {
    L->analysed = false;
    L->have_vals = L->have_rhs = L->solved = false;
    L->row_x.clear();
    L->row_y.clear();
  }
  L->rank = n;
  return PG_OK;
}

extern "C" int pg_lu_set_row_coords(pg_lu *L, const double *xy) {
  PG_CHECK_ARG(L, "pg_lu_set_row_coords: NULL handle");
  std::vector<double> nx, ny;
  if (xy) {
    PG_CHECK_ARG(L->rank > 0, "pg_lu_set_row_coords: set_rank first");
    nx.resize(L->rank);
    ny.resize(L->rank);
    for (int64_t i = 0; i < L->rank; ++i) {
      nx[i] = xy[2 * i];
      ny[i] = xy[2 * i + 1];
    }
  }
  if (nx == L->row_x && ny == L->row_y) return PG_OK;
  L->row_x.swap(nx);
  L->row_y.swap(ny);
  L->analysed = false;
  return PG_OK;
}

extern "C" int pg_lu_set_csr(pg_lu *L, const int32_t *row_ptr,
                             const int32_t *col_ind, const double *vals,
                             int ptr_kind) {
  PG_CHECK_ARG(L && row_ptr && col_ind && vals, "pg_lu_set_csr: NULL arg");
  PG_CHECK_ARG(L->rank > 0, "pg_lu_set_csr: set_rank first");
  const int64_t n = L->rank;
  cudaStream_t st = stream();
  std::vector<int32_t> hrp, hci;
  if (ptr_kind == PG_DEVICE) {
    hrp.resize(n + 1);
    PG_CUDA(cudaMemcpyAsync(hrp.data(), row_ptr, (n + 1) * sizeof(int32_t),
                            cudaMemcpyDeviceToHost, st));
    PG_CUDA(cudaStreamSynchronize(st));
    PG_CHECK_ARG(hrp[n] >= 0, "pg_lu_set_csr: bad row_ptr");
    hci.resize(hrp[n]);
    PG_CUDA(cudaMemcpyAsync(hci.data(), col_ind, hci.size() * sizeof(int32_t),
                            cudaMemcpyDeviceToHost, st));
    PG_CUDA(cudaStreamSynchronize(st));
  } else {
    PG_CHECK_ARG(row_ptr[n] >= 0, "pg_lu_set_csr: bad row_ptr");
    hrp.assign(row_ptr, row_ptr + n + 1);
    hci.assign(col_ind, col_ind + row_ptr[n]);
  }
  const int64_t n_src = hrp[n];
  const bool same = L->analysed && L->eqn_pattern == 0 && hrp == L->raw_rp &&
                    hci == L->raw_ci;
  PG_CUDA(L->rp_st.upload(hrp));
  PG_CUDA(L->ci_st.upload(hci));
  if (ptr_kind == PG_DEVICE) {
    PG_CUDA(L->vals_st.reserve(n_src));
    PG_CUDA(cudaMemcpyAsync(L->vals_st.p, vals, n_src * sizeof(double),
                            cudaMemcpyDeviceToDevice, st));
  } else {
    PG_CUDA(L->vals_st.upload(vals, n_src));
  }
  if (!same) {
    const bool xy = (int64_t)L->row_x.size() == n;
    int rc = analyse_and_upload(L, hrp.data(), hci.data(),
                                xy ? L->row_x.data() : nullptr,
                                xy ? L->row_y.data() : nullptr);
    if (rc) return rc;
    L->raw_rp.swap(hrp);
    L->raw_ci.swap(hci);
    L->eqn_pattern = 0;
  }
  L->m_rp = L->rp_st.p;
  L->m_ci = L->ci_st.p;
  L->m_vals = L->vals_st.p;
  L->have_vals = true;
  L->factored = false;
  return PG_OK;
}

extern "C" int pg_lu_set_eqn(pg_lu *L, const pg_eqn *e) {
  PG_CHECK_ARG(L && e, "pg_lu_set_eqn: NULL arg");
  PG_CHECK_ARG(!e->momentum, "pg_lu_set_eqn: a momentum equation has two "
                             "right-hand sides");
  const int64_t n = e->p.n;
  if (L->rank != n) {
    L->rank = n;
    L->analysed = false;
  }
  if (!L->analysed || L->eqn_pattern != e->pattern_id) {
    const pg::HostMesh &hm = e->mesh->h;
    const bool xy = n == hm.n_cells;
    int rc = analyse_and_upload(L, e->p.row_ptr.data(), e->p.col_ind.data(),
                                xy ? hm.cx.data() : nullptr,
                                xy ? hm.cy.data() : nullptr);
    if (rc) return rc;
    L->eqn_pattern = e->pattern_id;
    L->raw_rp.clear();
    L->raw_ci.clear();
  }
  L->m_rp = e->row_ptr.p;
  L->m_ci = e->col_ind.p;
  L->m_vals = e->vals.p;
  // the solver receives -rhs_ (FiniteVolumeEquation.tpp:73)
  cudaStream_t st = stream();
  k_lu_scale<<<grid_of(n, 256), 256, 0, st>>>((int)n, e->rhs.p, -1.0, L->b.p);
  count_launches(1);
  PG_CUDA(cudaGetLastError());
  L->have_vals = L->have_rhs = true;
  L->factored = false;
  return PG_OK;
}

extern "C" int pg_lu_set_rhs(pg_lu *L, const double *rhs, int ptr_kind) {
  PG_CHECK_ARG(L && rhs, "pg_lu_set_rhs: NULL arg");
  PG_CHECK_ARG(L->analysed, "pg_lu_set_rhs: set the matrix first");
  PG_CUDA(copy_in(L->b.p, rhs, L->s.n * sizeof(double), ptr_kind));
  L->have_rhs = true;
  return PG_OK;
}

extern "C" int pg_lu_solve(pg_lu *L, pg_lu_stats *stats) {
  PG_CHECK_ARG(L, "pg_lu_solve: NULL handle");
  PG_CHECK_ARG(L->analysed && L->have_vals && L->have_rhs,
               "pg_lu_solve: matrix and rhs must be set first");
  if (!L->factored) {
    int rc = factor(L, L->m_vals, stream());
    if (rc) return rc;
  }
  int rc = solve_now(L);
  float fms = 0.f;
  if (cudaEventElapsedTime(&fms, L->ev[0], L->ev[1]) == cudaSuccess)
    L->factor_ms = fms;
  else
    cudaGetLastError();
  if (stats) {
    const LuSymbolic &s = L->s;
    stats->n_fronts = (int)s.fronts.size();
    stats->n_heights = s.n_heights;
    stats->max_front = s.max_m;
    stats->replaced_pivots = L->replaced;
    stats->factor_entries = s.factor_nnz;
    stats->flops = s.flops;
    stats->analyse_ms = L->analyse_ms;
    stats->factor_ms = L->factor_ms;
    stats->solve_ms = L->solve_ms;
    stats->rel_residual = L->rel_residual;
  }
  return rc;
}

extern "C" int pg_lu_get_x(const pg_lu *L, double *x, int ptr_kind) {
  PG_CHECK_ARG(L && x, "pg_lu_get_x: NULL arg");
  PG_CHECK_ARG(L->solved, "pg_lu_get_x: nothing solved");
  PG_CUDA(copy_out(x, L->x.p, L->s.n * sizeof(double), ptr_kind));
  PG_CUDA(cudaStreamSynchronize(stream()));
  return PG_OK;
}

extern "C" int pg_lu_analyse_pattern(int64_t n, const int32_t *row_ptr,
                                     const int32_t *col_ind, const double *xy,
                                     int leaf, int64_t *sizes, int32_t *perm,
                                     int32_t *fronts, int32_t *fidx) {
  PG_CHECK_ARG(row_ptr && col_ind && sizes, "pg_lu_analyse_pattern: NULL arg");
  std::vector<double> x, y;
  if (xy) {
    x.resize(n);
    y.resize(n);
    for (int64_t i = 0; i < n; ++i) {
      x[i] = xy[2 * i];
      y[i] = xy[2 * i + 1];
    }
  }
  LuSymbolic s;
  int rc = lu_analyse(n, row_ptr, col_ind, xy ? x.data() : nullptr,
                      xy ? y.data() : nullptr, leaf > 0 ? leaf : 64, s);
  if (rc) return rc;
  sizes[0] = (int64_t)s.fronts.size();
  sizes[1] = (int64_t)s.fidx.size();
  sizes[2] = s.n_heights;
  sizes[3] = s.max_m;
  if (perm) std::copy(s.perm.begin(), s.perm.end(), perm);
  if (fronts)
    for (size_t t = 0; t < s.fronts.size(); ++t) {
      fronts[4 * t] = s.fronts[t].s0;
      fronts[4 * t + 1] = s.fronts[t].k;
      fronts[4 * t + 2] = s.fronts[t].m;
      fronts[4 * t + 3] = s.fronts[t].parent;
    }
  if (fidx) std::copy(s.fidx.begin(), s.fidx.end(), fidx);
  return PG_OK;
}

namespace pg {

int lu_inverse_setup(int64_t n, const int32_t *row_ptr, const int32_t *col_ind,
                     pg_lu **out) {
  *out = nullptr;
  pg_lu *L = nullptr;
  int rc = pg_lu_create(&L);
  if (rc) return rc;
  L->rank = n;
  // small leaves: the pivot steps of one height run one after another, and
  // a 16-vertex leaf has at most 16 of them (a coarse matrix on a 32 x 64
  // grid of subdomains: 138 steps over 8 heights instead of 170 over 6, and
  // a quarter of the flops)
  rc = analyse_and_upload(L, row_ptr, col_ind, nullptr, nullptr, 16);
  if (rc || L->s.max_m > kLuSmallM) {
    pg_lu_destroy(L);
    return rc;
  }
  const size_t nn = (size_t)n * n;
  cudaError_t e = L->inv_y.reserve(nn);
  if (e == cudaSuccess) e = L->inv_cp.reserve((size_t)std::max<int64_t>(L->s.cpool, 1) * n);
  if (e == cudaSuccess) e = L->iperm.upload(L->s.iperm);
  if (e == cudaSuccess) e = L->pool32.reserve(L->s.pool);
  {
    const size_t smem = ((size_t)kLuSmallM * kLuSmallM +
                         (size_t)kLuSmallM * kInvCols) * sizeof(float);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_lu_inv_fwd,
                               cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)smem);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_lu_inv_bwd,
                               cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)smem);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(stream());
  if (e != cudaSuccess) {
    pg_lu_destroy(L);
    return cuda_fail(e, "lu_inverse_setup", __FILE__, __LINE__);
  }
  *out = L;
  return PG_OK;
}

int lu_inverse_launches(const pg_lu *L) { return L->inv_launches; }
bool lu_inverse_captured(const pg_lu *L) { return L->inv_captured; }
void lu_inverse_set_captured(pg_lu *L) { L->inv_captured = true; }

int lu_inverse_run(pg_lu *L, const double *vals, float *out, cudaStream_t st) {
  const LuSymbolic &s = L->s;
  const uint64_t before = launch_count();
  int rc = factor(L, vals, st, true);
  if (rc) return rc;
  LuArgs a = args_of(L);
  const int n = (int)s.n;
  const int tiles = (n + kInvCols - 1) / kInvCols;
  for (int h = 0; h < s.n_heights; ++h) {
    const int nf = s.h_all_ptr[h + 1] - s.h_all_ptr[h];
    const int mm = s.h_maxm[h];
    const size_t smem = ((size_t)mm * mm + (size_t)mm * kInvCols) * sizeof(float);
    k_lu_inv_fwd<<<dim3(nf, tiles), kInvCols, smem, st>>>(
        L->h_all.p + s.h_all_ptr[h], a, L->pool32.p, n, L->inv_y.p, L->inv_cp.p);
  }
  for (int h = s.n_heights - 1; h >= 0; --h) {
    const int nf = s.h_all_ptr[h + 1] - s.h_all_ptr[h];
    const int mm = s.h_maxm[h];
    const size_t smem = ((size_t)mm * mm + (size_t)mm * kInvCols) * sizeof(float);
    k_lu_inv_bwd<<<dim3(nf, tiles), kInvCols, smem, st>>>(
        L->h_all.p + s.h_all_ptr[h], a, L->pool32.p, n, L->inv_y.p);
  }
  const int64_t nn = (int64_t)n * n;
  k_lu_inv_out<<<(int)((nn + 255) / 256), 256, 0, st>>>(n, L->iperm.p,
                                                         L->inv_y.p, out);
  count_launches(2 * s.n_heights + 1);
  L->inv_launches = (int)(launch_count() - before);
  PG_CUDA(cudaGetLastError());
  return PG_OK;
}

}  // namespace pg
