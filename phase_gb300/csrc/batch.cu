// Batched BiCGStab kernels: many independent systems stacked block-
// diagonally in one permuted CSR, each with its own scalars (KScalars
// array) and its own convergence.  The row space of every system is cut
// into tiles of rows; one CTA owns one tile, so a CTA touches one system
// only and returns at once when that system has stopped.  Dot products are
// reduced per system: each tile writes its partial, and the last tile of a
// system to finish (per-system ticket) sums that system's partials in tile
// order (deterministic) and runs the system's scalar recurrence, exactly as
// the single-system kernels do (kernels.cu).
//
// Reliable updates run on the device too: a system whose recursive residual
// meets the tolerance, drops by kDelta2 since its last replacement, or
// breaks down pauses (done = 1) with a pending action; the fix-up kernel at
// the end of the chunk computes its FP64 true residual and confirms
// convergence, replaces the recursive residual, or restarts the iteration
// with a fresh shadow residual.  The condition kernel then decides, on the
// device, whether the CUDA graph's WHILE node runs another chunk: the whole
// batched solve is one graph launch.
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/phase_gb300.h"
#include "kernels.cuh"

namespace pg {

namespace {

enum { kActNone = 0, kActConfirm = 1, kActRestart = 2, kActReplace = 3 };
constexpr double kBatchDelta2 = 1e-4;
constexpr int kBatchMaxRestarts = 50;

__device__ __forceinline__ double warp_sum_b(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ bool fin(double v) { return isfinite(v); }

// Per-system reduction of ND values; true in the system's last tile, whose
// threads all hold tot[].
template <int ND>
__device__ bool sys_reduce(double (&v)[ND], int sys, int tile,
                           const BatchTiles &T, const BatchRed &R,
                           double (&tot)[ND]) {
  __shared__ double sh[ND][32];
  __shared__ bool is_last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int k = 0; k < ND; ++k) {
    const double s = warp_sum_b(v[k]);
    if (lane == 0) sh[k][warp] = s;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < ND; ++k) {
      double s = 0.;
      for (int i = 0; i < nw; ++i) s += sh[k][i];
      R.partials[(size_t)k * R.n_tiles + tile] = s;
    }
    __threadfence();
    const unsigned cnt = (unsigned)(T.tile_ptr[sys + 1] - T.tile_ptr[sys]);
    const unsigned t = atomicAdd(&R.tickets[sys], 1u);
    is_last = t == cnt - 1;
  }
  __syncthreads();
  if (!is_last) return false;
  __threadfence();
  const int t0 = T.tile_ptr[sys], t1 = T.tile_ptr[sys + 1];
#pragma unroll
  for (int k = 0; k < ND; ++k) {
    double s = 0.;
    for (int i = t0 + threadIdx.x; i < t1; i += blockDim.x)
      s += __ldcg(&R.partials[(size_t)k * R.n_tiles + i]);
    s = warp_sum_b(s);
    __syncthreads();
    if (lane == 0) sh[k][warp] = s;
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < ND; ++k) {
    double s = 0.;
    for (int i = 0; i < nw; ++i) s += sh[k][i];
    tot[k] = s;
  }
  if (threadIdx.x == 0) R.tickets[sys] = 0u;
  return true;
}

__device__ __forceinline__ double row_dot_b(const int32_t *__restrict__ rp,
                                            const int32_t *__restrict__ ci,
                                            const double *__restrict__ val,
                                            const double *__restrict__ x,
                                            int i) {
  double s = 0.;
  for (int j = rp[i]; j < rp[i + 1]; ++j) s += val[j] * x[ci[j]];
  return s;
}

// r = b - A x (x NULL: r = b); rh = r; p = v = 0; per-system rho = rr,
// bb = <b, b>; systems with init[sys] == 0 are left alone
__global__ void k_b_init(BatchTiles T, BatchRed R, const int32_t *rp,
                         const int32_t *ci, const double *val, const double *b,
                         const double *x, double *r, double *rh, double *p,
                         double *v, KScalars *sc, const int *init) {
  const int tile = blockIdx.x, sys = T.tile_sys[tile];
  if (!init[sys]) return;
  double acc[2] = {0., 0.};
  for (int i = T.tile_r0[tile] + threadIdx.x; i < T.tile_r1[tile]; i += blockDim.x) {
    const double ri = x ? b[i] - row_dot_b(rp, ci, val, x, i) : b[i];
    r[i] = ri;
    rh[i] = ri;
    p[i] = 0.;
    v[i] = 0.;
    acc[0] += ri * ri;
    acc[1] += b[i] * b[i];
  }
  double tot[2];
  if (sys_reduce<2>(acc, sys, tile, T, R, tot) && threadIdx.x == 0) {
    KScalars *s = sc + sys;
    s->rr = tot[0];
    s->rr_true = tot[0];
    s->rr_ref = tot[0];
    s->action = kActNone;
    s->restarts = 0;
    s->bb = tot[1];
    s->rho = tot[0];
    s->rho_prev = 1.;
    s->alpha = s->omega = 1.;
    s->beta = tot[0];
    s->status = PG_OK;
    s->done = 0;
    if (!fin(tot[0]) || !fin(tot[1])) {
      s->status = PG_NON_FINITE;
      s->done = 1;
    } else if (tot[0] <= s->tol2 * tot[1]) {
      s->done = 1;  // already converged (or b = 0)
    }
  }
}

__global__ void k_b_spmv_v(BatchTiles T, BatchRed R, SolverDev d,
                           const double *val, const double *ph, double *v,
                           const double *rh, KScalars *sc) {
  const int tile = blockIdx.x, sys = T.tile_sys[tile];
  if (sc[sys].done) return;
  double acc[1] = {0.};
  for (int i = T.tile_r0[tile] + threadIdx.x; i < T.tile_r1[tile]; i += blockDim.x) {
    const double vi = row_dot_b(d.prp, d.pci, val, ph, i);
    v[i] = vi;
    acc[0] += rh[i] * vi;
  }
  double tot[1];
  if (sys_reduce<1>(acc, sys, tile, T, R, tot) && threadIdx.x == 0) {
    KScalars *s = sc + sys;
    s->rv = tot[0];
    if (!fin(tot[0])) {
      s->status = PG_NON_FINITE;
      s->done = 1;
    } else if (tot[0] == 0.) {
      s->status = PG_BREAKDOWN;
      s->done = 1;
      s->action = kActRestart;
    } else {
      s->alpha = s->rho / tot[0];
    }
  }
}

__global__ void k_b_spmv_t(BatchTiles T, BatchRed R, SolverDev d,
                           const double *val, const double *sh, double *t,
                           const double *s_, KScalars *sc) {
  const int tile = blockIdx.x, sys = T.tile_sys[tile];
  if (sc[sys].done) return;
  double acc[2] = {0., 0.};
  for (int i = T.tile_r0[tile] + threadIdx.x; i < T.tile_r1[tile]; i += blockDim.x) {
    const double ti = row_dot_b(d.prp, d.pci, val, sh, i);
    t[i] = ti;
    acc[0] += ti * ti;
    acc[1] += ti * s_[i];
  }
  double tot[2];
  if (sys_reduce<2>(acc, sys, tile, T, R, tot) && threadIdx.x == 0) {
    KScalars *s = sc + sys;
    s->tt = tot[0];
    s->ts = tot[1];
    s->omega = tot[0] > 0. ? tot[1] / tot[0] : 0.;
  }
}

__global__ void k_b_update(BatchTiles T, BatchRed R, double *x, double *r,
                           const double *ph, const double *sh,
                           const double *s_, const double *t,
                           const double *rh, KScalars *sc) {
  const int tile = blockIdx.x, sys = T.tile_sys[tile];
  if (sc[sys].done) return;
  const double al = sc[sys].alpha, om = sc[sys].omega;
  double acc[2] = {0., 0.};
  for (int i = T.tile_r0[tile] + threadIdx.x; i < T.tile_r1[tile]; i += blockDim.x) {
    x[i] = x[i] + al * ph[i] + om * sh[i];
    const double ri = s_[i] - om * t[i];
    r[i] = ri;
    acc[0] += rh[i] * ri;
    acc[1] += ri * ri;
  }
  double tot[2];
  if (sys_reduce<2>(acc, sys, tile, T, R, tot) && threadIdx.x == 0) {
    KScalars *s = sc + sys;
    const double rho_new = tot[0];
    s->rr = tot[1];
    s->iter += 1;
    if (!fin(tot[0]) || !fin(tot[1])) {
      s->status = PG_NON_FINITE;
      s->done = 1;
    } else {
      if (om != 0. && s->rho != 0.) s->beta = (rho_new / s->rho) * (al / om);
      s->rho_prev = s->rho;
      s->rho = rho_new;
      if (tot[1] <= s->tol2 * s->bb) {
        s->status = PG_OK;
        s->done = 1;
        s->action = kActConfirm;
      } else if (s->iter >= s->max_iter) {
        s->status = PG_MAX_ITERS;
        s->done = 1;
      } else if (rho_new == 0. || om == 0.) {
        s->status = PG_BREAKDOWN;
        s->done = 1;
        s->action = kActRestart;
      } else if (tot[1] < kBatchDelta2 * s->rr_ref) {
        s->done = 1;
        s->action = kActReplace;
      }
    }
  }
}

__global__ void k_b_fix(BatchTiles T, BatchRed R, const int32_t *rp,
                        const int32_t *ci, const double *val, const double *b,
                        const double *x, double *r, double *rh, double *p,
                        double *v, KScalars *sc) {
  const int tile = blockIdx.x, sys = T.tile_sys[tile];
  const int act = sc[sys].action;
  if (act == kActNone) return;
  double acc[2] = {0., 0.};
  for (int i = T.tile_r0[tile] + threadIdx.x; i < T.tile_r1[tile]; i += blockDim.x) {
    const double ri = b[i] - row_dot_b(rp, ci, val, x, i);
    r[i] = ri;
    if (act == kActRestart) {
      rh[i] = ri;
      p[i] = 0.;
      v[i] = 0.;
      acc[0] += ri * ri;
    } else {
      acc[0] += rh[i] * ri;
    }
    acc[1] += ri * ri;
  }
  double tot[2];
  if (sys_reduce<2>(acc, sys, tile, T, R, tot) && threadIdx.x == 0) {
    KScalars *s = sc + sys;
    s->rr_true = tot[1];
    s->rr_ref = tot[1];
    s->rr = tot[1];
    s->action = kActNone;
    if (!fin(tot[0]) || !fin(tot[1])) {
      s->status = PG_NON_FINITE;
      s->done = 1;
    } else if (tot[1] <= s->tol2 * s->bb) {
      s->status = PG_OK;
      s->done = 1;
    } else if (s->iter >= s->max_iter) {
      s->status = PG_MAX_ITERS;
      s->done = 1;
    } else if (act == kActRestart) {
      if (++s->restarts > kBatchMaxRestarts) {
        s->status = PG_BREAKDOWN;
        s->done = 1;
      } else {
        s->rho = tot[1];
        s->rho_prev = 1.;
        s->alpha = s->omega = 1.;
        s->beta = tot[1];
        s->status = PG_OK;
        s->done = 0;
      }
    } else if (tot[0] == 0. || s->omega == 0. || s->rho_prev == 0.) {
      s->action = kActRestart;  // handled at the next fix-up
      s->done = 1;
    } else {
      s->beta = (tot[0] / s->rho_prev) * (s->alpha / s->omega);
      s->rho = tot[0];
      s->status = PG_OK;
      s->done = 0;
    }
  }
}

// rr_true = ||b - A x||^2 per system; with sel != NULL only the systems
// with sel[sys] != 0, and then r = b - A x and the residual replacement
// (rho, beta from the new r, the search directions kept)
__global__ void k_b_true_residual(BatchTiles T, BatchRed R, const int32_t *rp,
                                  const int32_t *ci, const double *val,
                                  const double *b, const double *x, double *r,
                                  const double *rh, KScalars *sc,
                                  const int *sel) {
  const int tile = blockIdx.x, sys = T.tile_sys[tile];
  if (sel && !sel[sys]) return;
  double acc[2] = {0., 0.};
  for (int i = T.tile_r0[tile] + threadIdx.x; i < T.tile_r1[tile]; i += blockDim.x) {
    const double ri = b[i] - row_dot_b(rp, ci, val, x, i);
    acc[0] += ri * ri;
    if (sel) {
      r[i] = ri;
      acc[1] += rh[i] * ri;
    }
  }
  double tot[2];
  if (sys_reduce<2>(acc, sys, tile, T, R, tot) && threadIdx.x == 0) {
    KScalars *s = sc + sys;
    s->rr_true = tot[0];
    if (sel) {
      s->rr = tot[0];
      s->done = 0;
      s->status = PG_OK;
      if (!fin(tot[0]) || !fin(tot[1])) {
        s->status = PG_NON_FINITE;
        s->done = 1;
      } else if (tot[1] == 0. || s->omega == 0. || s->rho_prev == 0.) {
        s->status = PG_BREAKDOWN;
        s->done = 1;
      } else {
        s->beta = (tot[1] / s->rho_prev) * (s->alpha / s->omega);
        s->rho = tot[1];
      }
    }
  }
}

// End of a chunk: run another one while a system is still iterating and
// the chunk budget is not spent (the loop always terminates: every system
// stops at its max_iter, and the budget bounds the chunks regardless).
__global__ void k_b_check(int n_sys, const KScalars *sc, int *chunks,
                          int max_chunks, cudaGraphConditionalHandle h) {
  __shared__ int any;
  if (threadIdx.x == 0) any = 0;
  __syncthreads();
  int mine = 0;
  for (int s = threadIdx.x; s < n_sys; s += blockDim.x)
    mine |= !sc[s].done || sc[s].action != kActNone;
  if (mine) atomicOr(&any, 1);
  __syncthreads();
  if (threadIdx.x == 0) {
    const int c = *chunks + 1;
    *chunks = c;
    cudaGraphSetConditional(h, (any && c < max_chunks) ? 1u : 0u);
  }
}

}  // namespace

void launch_b_init(const BatchTiles &T, const BatchRed &R, int block,
                   const int32_t *rp, const int32_t *ci, const double *val,
                   const double *b, const double *x, double *r, double *rh,
                   double *p, double *v, KScalars *sc, const int *init,
                   cudaStream_t st) {
  k_b_init<<<T.n_tiles, block, 0, st>>>(T, R, rp, ci, val, b, x, r, rh, p, v,
                                        sc, init);
  count_launches(1);
}
void launch_b_spmv_v(const BatchTiles &T, const BatchRed &R, int block,
                     const SolverDev &d, const double *val,
                     const double *ph, double *v, const double *rh,
                     KScalars *sc, cudaStream_t st) {
  k_b_spmv_v<<<T.n_tiles, block, 0, st>>>(T, R, d, val, ph, v, rh, sc);
  count_launches(1);
}
void launch_b_spmv_t(const BatchTiles &T, const BatchRed &R, int block,
                     const SolverDev &d, const double *val,
                     const double *sh, double *t, const double *s,
                     KScalars *sc, cudaStream_t st) {
  k_b_spmv_t<<<T.n_tiles, block, 0, st>>>(T, R, d, val, sh, t, s, sc);
  count_launches(1);
}
void launch_b_update(const BatchTiles &T, const BatchRed &R, int block,
                     double *x, double *r, const double *ph, const double *sh,
                     const double *s, const double *t, const double *rh,
                     KScalars *sc, cudaStream_t st) {
  k_b_update<<<T.n_tiles, block, 0, st>>>(T, R, x, r, ph, sh, s, t, rh, sc);
  count_launches(1);
}
void launch_b_true_residual(const BatchTiles &T, const BatchRed &R, int block,
                            const int32_t *rp, const int32_t *ci,
                            const double *val, const double *b,
                            const double *x, double *r, const double *rh,
                            KScalars *sc, const int *sel, cudaStream_t st) {
  k_b_true_residual<<<T.n_tiles, block, 0, st>>>(T, R, rp, ci, val, b, x, r,
                                                 rh, sc, sel);
  count_launches(1);
}
void launch_b_fix(const BatchTiles &T, const BatchRed &R, int block,
                  const int32_t *rp, const int32_t *ci, const double *val,
                  const double *b, const double *x, double *r, double *rh,
                  double *p, double *v, KScalars *sc, cudaStream_t st) {
  k_b_fix<<<T.n_tiles, block, 0, st>>>(T, R, rp, ci, val, b, x, r, rh, p, v,
                                       sc);
  count_launches(1);
}
void launch_b_check(int n_sys, const KScalars *sc, int *chunks,
                    int max_chunks, cudaGraphConditionalHandle h,
                    cudaStream_t st) {
  k_b_check<<<1, 256, 0, st>>>(n_sys, sc, chunks, max_chunks, h);
  count_launches(1);
}

}  // namespace pg
