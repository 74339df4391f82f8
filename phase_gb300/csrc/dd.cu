// Krylov kernels of the mixed-precision solver in float-float arithmetic
// (dd.cuh): SpMV with the fused dot products, the BiCGStab x/r update,
// residual replacement, and the conversions to and from the FP64 solution.
//
// Every per-element operation runs on the FP32 pipes; FP64 instructions
// appear only in the per-block partial sums of the dot products, in the
// last block's scalar recurrences, and in the conversion kernels that run
// once per reliable update (FP64 residual in, float pairs out).  The
// reduction order is fixed (warp tree, block tree, last-block sum of the
// per-block partials), so results are deterministic, as in kernels.cu.
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/phase_gb300.h"
#include "dd.cuh"
#include "kernels.cuh"
#include "tma.cuh"

namespace pg {

namespace {

__device__ __forceinline__ DdAcc shfl_xor(const DdAcc &a, int o) {
  return DdAcc{__shfl_xor_sync(0xffffffffu, a.s, o),
               __shfl_xor_sync(0xffffffffu, a.c, o)};
}

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Grid reduction of ND compensated sums.  The warp and block trees merge
// float-float accumulators; one FP64 partial per block goes to the
// workspace; the last block to finish sums the partials in FP64.  Returns
// true in the last block, whose threads all hold tot[].
template <int ND>
__device__ bool grid_reduce_dd(DdAcc (&v)[ND], const RedWork &w,
                               double (&tot)[ND]) {
  __shared__ DdAcc sh[ND][kVecBlock / 32];
  __shared__ double shd[ND][kVecBlock / 32];
  __shared__ bool is_last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nw = blockDim.x >> 5;
#pragma unroll
  for (int k = 0; k < ND; ++k) {
    DdAcc a = v[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) dd_acc_merge(a, shfl_xor(a, o));
    if (lane == 0) sh[k][warp] = a;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < ND; ++k) {
      DdAcc a = sh[k][0];
      for (int i = 1; i < nw; ++i) dd_acc_merge(a, sh[k][i]);
      w.partials[k * w.grid + blockIdx.x] = dd_acc_to_double(a);
    }
    __threadfence();
    unsigned int t = atomicAdd(w.ticket, 1u);
    is_last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!is_last) return false;
  __threadfence();
#pragma unroll
  for (int k = 0; k < ND; ++k) {
    double s = 0.;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x)
      s += __ldcg(&w.partials[k * w.grid + i]);
    s = warp_sum_d(s);
    if (lane == 0) shd[k][warp] = s;
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < ND; ++k) {
    double s = 0.;
    for (int i = 0; i < nw; ++i) s += shd[k][i];
    tot[k] = s;
  }
  if (threadIdx.x == 0) *w.ticket = 0u;
  return true;
}

__device__ __forceinline__ bool finite_d(double v) { return isfinite(v); }

// The BiCGStab recurrences of the float-float kernels (last block,
// thread 0): after the x / r update (tot = {<rhat, r>, <r, r>}), after
// v = A phat (alpha from <rhat, v>), after t = A shat (omega)
__device__ __forceinline__ void dd_update_scalars(KScalars *sc, const double (&tot)[2]) {
  const double rho_new = tot[0], alv = sc->alpha, omv = sc->omega;
  sc->rr = tot[1];
  sc->iter += 1;
  if (!finite_d(tot[0]) || !finite_d(tot[1])) {
    sc->status = PG_NON_FINITE;
    sc->done = 1;
  } else {
    if (omv != 0. && sc->rho != 0.)
      sc->beta = (rho_new / sc->rho) * (alv / omv);
    sc->beta_dd = dd_from(sc->beta);
    sc->rho_prev = sc->rho;
    sc->rho = rho_new;
    if (tot[1] <= sc->tol2 * sc->bb) {
      sc->status = PG_OK;
      sc->done = 1;
    } else if (sc->iter >= sc->max_iter) {
      sc->status = PG_MAX_ITERS;
      sc->done = 1;
    } else if (rho_new == 0. || omv == 0.) {
      sc->status = PG_BREAKDOWN;
      sc->done = 1;
    }
  }
}
__device__ __forceinline__ void dd_spmv_v_scalars(KScalars *sc, double rv) {
  sc->rv = rv;
  if (!finite_d(rv)) {
    sc->status = PG_NON_FINITE;
    sc->done = 1;
  } else if (rv == 0.) {
    sc->status = PG_BREAKDOWN;
    sc->done = 1;
  } else {
    sc->alpha = sc->rho / rv;
    sc->alpha_dd = dd_from(sc->alpha);
  }
}
__device__ __forceinline__ void dd_spmv_t_scalars(KScalars *sc, const double (&tot)[2]) {
  sc->tt = tot[0];
  sc->ts = tot[1];
  sc->omega = tot[0] > 0. ? tot[1] / tot[0] : 0.;
  sc->omega_dd = dd_from(sc->omega);
}

__device__ __forceinline__ float2 row_dot_dd(const int32_t *__restrict__ rp,
                                             const int32_t *__restrict__ ci,
                                             const float2 *__restrict__ val,
                                             const float2 *__restrict__ x,
                                             int i) {
  DdAcc a{0.f, 0.f};
  const int b = rp[i], e = rp[i + 1];
  for (int j = b; j < e; ++j) dd_acc_fma(a, val[j], x[ci[j]]);
  return dd_value(a);
}

__global__ void k_dd_split(int64_t n, const double *__restrict__ src,
                           double scale, float2 *__restrict__ dst) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = dd_from(src[i] * scale);
}

__global__ void k_dd_join(int n, const float2 *__restrict__ src, double scale,
                          double *__restrict__ dst) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += gridDim.x * blockDim.x)
    dst[i] = dd_to_double(src[i]) * scale;
}

__global__ void k_dd_fold(int n, double *__restrict__ x64,
                          float2 *__restrict__ xw, double inv_scale) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += gridDim.x * blockDim.x) {
    x64[i] += dd_to_double(xw[i]) * inv_scale;
    xw[i] = make_float2(0.f, 0.f);
  }
}

// r = dd(r64 * scale); restart: rhat = r, p = v = 0, rho = <r, r>;
// otherwise residual replacement: rho_{i+1} = <rhat, r>, beta_i from it
__global__ void __launch_bounds__(kVecBlock)
k_dd_set_r(int n, const double *__restrict__ r64, double scale,
           float2 *__restrict__ r, float2 *__restrict__ rh,
           float2 *__restrict__ p, float2 *__restrict__ v, int restart,
           KScalars *sc, RedWork w) {
  DdAcc acc[2] = {{0.f, 0.f}, {0.f, 0.f}};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += gridDim.x * blockDim.x) {
    const float2 ri = dd_from(r64[i] * scale);
    r[i] = ri;
    float2 rhi;
    if (restart) {
      rh[i] = ri;
      p[i] = make_float2(0.f, 0.f);
      v[i] = make_float2(0.f, 0.f);
      rhi = ri;
    } else {
      rhi = rh[i];
    }
    dd_acc_fma(acc[0], rhi, ri);
    dd_acc_fma(acc[1], ri, ri);
  }
  double tot[2];
  if (grid_reduce_dd<2>(acc, w, tot) && threadIdx.x == 0) {
    sc->rr = tot[1];
    sc->done = 0;
    sc->status = PG_OK;
    if (!finite_d(tot[0]) || !finite_d(tot[1])) {
      sc->status = PG_NON_FINITE;
      sc->done = 1;
    } else if (restart) {
      sc->rho = tot[1];
      sc->rho_prev = 1.;
      sc->alpha = sc->omega = 1.;
      sc->beta = tot[1];
      if (tot[1] == 0.) sc->done = 1;
    } else if (tot[0] == 0. || sc->omega == 0. || sc->rho_prev == 0.) {
      sc->status = PG_BREAKDOWN;
      sc->done = 1;
    } else {
      sc->beta = (tot[0] / sc->rho_prev) * (sc->alpha / sc->omega);
      sc->rho = tot[0];
    }
    sc->alpha_dd = dd_from(sc->alpha);
    sc->omega_dd = dd_from(sc->omega);
    sc->beta_dd = dd_from(sc->beta);
  }
}

__global__ void __launch_bounds__(kVecBlock)
k_dd_spmv_v(SolverDev d, const float2 *__restrict__ val,
            const float2 *__restrict__ ph, float2 *__restrict__ v,
            const float2 *__restrict__ rh, KScalars *sc, RedWork w) {
  pdl_wait();
  if (sc->done) return;
  DdAcc acc[1] = {{0.f, 0.f}};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < d.n;
       i += gridDim.x * blockDim.x) {
    const float2 vi = row_dot_dd(d.prp, d.pci, val, ph, i);
    v[i] = vi;
    dd_acc_fma(acc[0], rh[i], vi);
  }
  double tot[1];
  if (grid_reduce_dd<1>(acc, w, tot) && threadIdx.x == 0) dd_spmv_v_scalars(sc, tot[0]);
}

__global__ void __launch_bounds__(kVecBlock)
k_dd_spmv_t(SolverDev d, const float2 *__restrict__ val,
            const float2 *__restrict__ sh, float2 *__restrict__ t,
            const float2 *__restrict__ s, KScalars *sc, RedWork w) {
  pdl_wait();
  if (sc->done) return;
  DdAcc acc[2] = {{0.f, 0.f}, {0.f, 0.f}};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < d.n;
       i += gridDim.x * blockDim.x) {
    const float2 ti = row_dot_dd(d.prp, d.pci, val, sh, i);
    t[i] = ti;
    dd_acc_fma(acc[0], ti, ti);
    dd_acc_fma(acc[1], ti, s[i]);
  }
  double tot[2];
  if (grid_reduce_dd<2>(acc, w, tot) && threadIdx.x == 0) dd_spmv_t_scalars(sc, tot);
}

__global__ void __launch_bounds__(kVecBlock)
k_dd_update(int n, float2 *__restrict__ x, float2 *__restrict__ r,
            const float2 *__restrict__ ph, const float2 *__restrict__ sh,
            const float2 *__restrict__ s, const float2 *__restrict__ t,
            const float2 *__restrict__ rh, KScalars *sc, RedWork w) {
  pdl_wait();
  if (sc->done) return;
  const float2 al = sc->alpha_dd, om = sc->omega_dd;
  DdAcc acc[2] = {{0.f, 0.f}, {0.f, 0.f}};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += gridDim.x * blockDim.x) {
    x[i] = dd_add(x[i], dd_add(dd_mul(al, ph[i]), dd_mul(om, sh[i])));
    const float2 ri = dd_sub(s[i], dd_mul(om, t[i]));
    r[i] = ri;
    dd_acc_fma(acc[0], rh[i], ri);
    dd_acc_fma(acc[1], ri, ri);
  }
  double tot[2];
  if (grid_reduce_dd<2>(acc, w, tot) && threadIdx.x == 0) dd_update_scalars(sc, tot);
}

// ---- streamed x / r update (bulk copies through shared memory, tma.cuh;
// the same per-element arithmetic as k_dd_update, each thread's sums in its
// tiles' order).  The SpMVs stay thread-per-row: their x gathers, not the
// matrix stream, set their time, and a tile ring's CTAs hide them worse. ----
constexpr int kUpdStages = 4;   // tiles in flight per CTA, x / r update

__global__ void __launch_bounds__(kTileN)
k_dd_update_tma(int n, float2 *__restrict__ x, float2 *__restrict__ r,
                const float2 *__restrict__ ph, const float2 *__restrict__ sh,
                const float2 *__restrict__ s, const float2 *__restrict__ t,
                const float2 *__restrict__ rh, KScalars *sc, RedWork w) {
  extern __shared__ __align__(128) uint8_t smem[];
  __shared__ __align__(8) uint64_t bar[kUpdStages];
  pdl_wait();
  if (sc->done) return;
  const float2 al = sc->alpha_dd, om = sc->omega_dd;
  const int tid = threadIdx.x, G = gridDim.x, blk = blockIdx.x;
  const int n_tiles = (n + kTileN - 1) / kTileN;
  const int m = blk < n_tiles ? (n_tiles - 1 - blk) / G + 1 : 0;
  constexpr int kStage = 6 * kTileN * 8;
  const void *const src[6] = {x, ph, sh, s, t, rh};
  if (tid == 0) {
    for (int b = 0; b < kUpdStages; ++b) mbar_init(&bar[b], 1);
    for (int k = 0; k < kUpdStages && k < m; ++k)
      issue_vec_tile<6>(smem + k * kStage, src, n, blk + k * G, &bar[k]);
  }
  __syncthreads();
  DdAcc acc[2] = {{0.f, 0.f}, {0.f, 0.f}};
  int k = 0;
  bool failed = false;
  for (; k < m; ++k) {
    const int b = k % kUpdStages;
    const bool ok = mbar_wait_bounded(&bar[b], w.err, (uint32_t)((k / kUpdStages) & 1));
    if (__syncthreads_or(!ok)) {
      failed = true;
      break;
    }
    const int j = blk + k * G;
    const int i = j * kTileN + tid;
    if (i < n) {
      const float2 *stg = reinterpret_cast<const float2 *>(smem + b * kStage);
      float2 xv, pv, shv, sv, tv, rhv;
      if (tid < tile_bulk_count(n, j)) {
        xv = stg[tid];
        pv = stg[kTileN + tid];
        shv = stg[2 * kTileN + tid];
        sv = stg[3 * kTileN + tid];
        tv = stg[4 * kTileN + tid];
        rhv = stg[5 * kTileN + tid];
      } else {
        xv = x[i];
        pv = ph[i];
        shv = sh[i];
        sv = s[i];
        tv = t[i];
        rhv = rh[i];
      }
      x[i] = dd_add(xv, dd_add(dd_mul(al, pv), dd_mul(om, shv)));
      const float2 ri = dd_sub(sv, dd_mul(om, tv));
      r[i] = ri;
      dd_acc_fma(acc[0], rhv, ri);
      dd_acc_fma(acc[1], ri, ri);
    }
    __syncthreads();  // stage b is free
    if (tid == 0 && k + kUpdStages < m) {
      fence_proxy_async();
      issue_vec_tile<6>(smem + b * kStage, src, n, blk + (k + kUpdStages) * G, &bar[b]);
    }
  }
  if (failed && tid == 0)  // the copies still in flight, before leaving
    for (int k2 = k + 1; k2 < m && k2 < k + kUpdStages; ++k2)
      mbar_wait_bounded(&bar[k2 % kUpdStages], nullptr, (uint32_t)((k2 / kUpdStages) & 1));
  double tot[2];
  if (grid_reduce_dd<2>(acc, w, tot) && threadIdx.x == 0) dd_update_scalars(sc, tot);
}

template <int MODE>
__global__ void k_dd_diag_apply(int n, const float2 *__restrict__ dinv,
                                const float2 *__restrict__ r,
                                float2 *__restrict__ pv,
                                const float2 *__restrict__ v,
                                float2 *__restrict__ z, const KScalars *sc) {
  if (sc && sc->done) return;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += gridDim.x * blockDim.x) {
    const float2 in = dd_pre_input(MODE, i, r, pv, v, sc);
    z[i] = dinv ? dd_mul(dinv[i], in) : in;
  }
}

inline int grid_of(int64_t n) {
  const int64_t g = (n + 255) / 256;
  return (int)(g < 1 ? 1 : g > 2432 ? 2432 : g);
}

}  // namespace

void launch_dd_split(int64_t n, const double *src, double scale, float2 *dst,
                     cudaStream_t st) {
  k_dd_split<<<grid_of(n), 256, 0, st>>>(n, src, scale, dst);
  count_launches(1);
}

void launch_dd_join(int n, const float2 *src, double scale, double *dst,
                    cudaStream_t st) {
  k_dd_join<<<grid_of(n), 256, 0, st>>>(n, src, scale, dst);
  count_launches(1);
}

void launch_dd_fold(int n, double *x64, float2 *xw, double inv_scale,
                    cudaStream_t st) {
  k_dd_fold<<<grid_of(n), 256, 0, st>>>(n, x64, xw, inv_scale);
  count_launches(1);
}

void launch_dd_set_r(int n, const double *r64, double scale, float2 *r,
                     float2 *rh, float2 *p, float2 *v, bool restart,
                     KScalars *sc, RedWork w, cudaStream_t st) {
  k_dd_set_r<<<w.grid, kVecBlock, 0, st>>>(n, r64, scale, r, rh, p, v,
                                           restart ? 1 : 0, sc, w);
  count_launches(1);
}

void launch_dd_spmv_v(const SolverDev &d, const float2 *val, const float2 *ph,
                      float2 *v, const float2 *rh, KScalars *sc, RedWork w,
                      cudaStream_t st) {
  launch_pdl(k_dd_spmv_v, w.grid, kVecBlock, 0, st, d, val, ph, v, rh, sc, w);
  count_launches(1);
}

void launch_dd_spmv_t(const SolverDev &d, const float2 *val, const float2 *sh,
                      float2 *t, const float2 *s, KScalars *sc, RedWork w,
                      cudaStream_t st) {
  launch_pdl(k_dd_spmv_t, w.grid, kVecBlock, 0, st, d, val, sh, t, s, sc, w);
  count_launches(1);
}

void launch_dd_update(int n, float2 *x, float2 *r, const float2 *ph,
                      const float2 *sh, const float2 *s, const float2 *t,
                      const float2 *rh, KScalars *sc, RedWork w,
                      cudaStream_t st) {
  if (stream_enabled() && n > 0 && aligned16(x) && aligned16(r) &&
      aligned16(ph) && aligned16(sh) && aligned16(s) && aligned16(t) &&
      aligned16(rh)) {
    constexpr size_t smem = kUpdStages * 6 * kTileN * 8;
    static bool attr = false;
    if (!attr) {
      cudaFuncSetAttribute(k_dd_update_tma,
                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      attr = true;
    }
    const int g = stream_grid((const void *)k_dd_update_tma, smem,
                              (n + kTileN - 1) / kTileN, w.grid);
    launch_pdl(k_dd_update_tma, g, kTileN, smem, st, n, x, r, ph, sh, s, t, rh, sc, w);
    count_launches(1);
    return;
  }
  launch_pdl(k_dd_update, w.grid, kVecBlock, 0, st, n, x, r, ph, sh, s, t, rh, sc, w);
  count_launches(1);
}

void launch_dd_diag_apply(int mode, int n, const float2 *dinv, const float2 *r,
                          float2 *pv, const float2 *v, float2 *z,
                          const KScalars *sc, cudaStream_t st) {
  if (mode == 0)
    k_dd_diag_apply<0><<<grid_of(n), 256, 0, st>>>(n, dinv, r, pv, v, z, sc);
  else if (mode == 1)
    k_dd_diag_apply<1><<<grid_of(n), 256, 0, st>>>(n, dinv, r, pv, v, z, sc);
  else
    k_dd_diag_apply<2><<<grid_of(n), 256, 0, st>>>(n, dinv, r, pv, v, z, sc);
  count_launches(1);
}

}  // namespace pg
