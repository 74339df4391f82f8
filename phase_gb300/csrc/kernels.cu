// CUDA kernels of libphase_gb300, written for sm_103a (GB300).
//
// The sparse pressure path is HBM-bandwidth bound and uses no tensor cores.
//  * Assembly: face-coloured, atomic-free scatter of fv::laplacian + src::div
//    into the CSR values and rhs (one launch per colour).
//  * Solver: values are gathered once per solve into a permuted CSR in which
//    every Schwarz subdomain is a contiguous, level-ordered row range.  ILU(0)
//    is factorised and applied per subdomain by one CTA that walks the level
//    schedule with a barrier between levels; the subdomain's factor and
//    vector are staged in shared memory for the triangular sweeps.
//  * BiCGStab: every dot product is fused into the kernel that produces its
//    operands (warp shuffle + block tree + last-block grid reduction in a
//    fixed order, so results are deterministic) and the scalar recurrences
//    (alpha, beta, omega, convergence) run on the device in the last block.
#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <cstdlib>

#include "../../include/phase_gb300.h"
#include <type_traits>

#include "kernels.cuh"
#include "tma.cuh"

namespace pg {

static std::atomic<uint64_t> g_launches{0};
void count_launches(int k) { g_launches.fetch_add((uint64_t)k, std::memory_order_relaxed); }
uint64_t launch_count() { return g_launches.load(std::memory_order_relaxed); }
bool pdl_enabled() {
  static const bool on = [] {
    const char *e = std::getenv("PG_PDL");
    return !(e && e[0] == '0');
  }();
  return on;
}

namespace {

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ bool finite(double v) { return isfinite(v); }

// Block-reduce ND values, store the block partials, and let the last block
// to finish reduce all partials (fixed order) into tot[].  Returns true in
// the last block only; tot[] is valid in all its threads.
template <int ND>
__device__ bool grid_reduce(double (&v)[ND], const RedWork &w,
                            double (&tot)[ND]) {
  __shared__ double sh[ND][kVecBlock / 32];
  __shared__ bool is_last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nw = blockDim.x >> 5;
#pragma unroll
  for (int k = 0; k < ND; ++k) {
    double s = warp_sum(v[k]);
    if (lane == 0) sh[k][warp] = s;
  }
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int k = 0; k < ND; ++k) {
      double s = lane < nw ? sh[k][lane] : 0.;
      s = warp_sum(s);
      if (lane == 0) w.partials[k * w.grid + blockIdx.x] = s;
    }
  }
  if (threadIdx.x == 0) {
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
    s = warp_sum(s);
    if (lane == 0) sh[k][warp] = s;
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < ND; ++k) {
    double s = 0.;
    for (int i = 0; i < nw; ++i) s += sh[k][i];
    tot[k] = s;
  }
  if (threadIdx.x == 0) *w.ticket = 0u;
  return true;
}

// ------------------------------------------------------------ assembly
// One launch per interior colour: no two faces of a colour share a cell,
// so every += below has a single writer in the launch.  Arithmetic uses
// explicitly rounded operations in the reference's order:
// coeff = (gamma * dot(r, Sf)) / |r|^2  (Laplacian.h:139-142, 55-58).
__global__ void k_assemble_interior(
    int nf, int off, const int32_t *__restrict__ cface,
    const int32_t *__restrict__ cl, const int32_t *__restrict__ cr,
    const double *__restrict__ dot_l, const double *__restrict__ dot_r,
    const double *__restrict__ msq, const int32_t *__restrict__ slot_lr,
    const int32_t *__restrict__ slot_rl, const int32_t *__restrict__ diag_l,
    const int32_t *__restrict__ diag_r, const double *__restrict__ sfl_x,
    const double *__restrict__ sfl_y, const double *__restrict__ sfr_x,
    const double *__restrict__ sfr_y, const double *__restrict__ gamma_face,
    double gamma_scalar, const double *__restrict__ u_face,
    double *__restrict__ vals, double *__restrict__ rhs) {
  const int k = off + blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= off + nf) return;
  const int f = cface[k];
  const int l = cl[k], r = cr[k];
  const double g = gamma_face ? gamma_face[f] : gamma_scalar;
  const double m2 = msq[k];
  const double c_l = __ddiv_rn(__dmul_rn(g, dot_l[k]), m2);
  const double c_r = __ddiv_rn(__dmul_rn(g, dot_r[k]), m2);
  // a side with cell -1 is not a fluid row (ghost-cell IB equations)
  if (l >= 0) {
    vals[slot_lr[k]] = __dadd_rn(vals[slot_lr[k]], c_l);
    vals[diag_l[k]] = __dadd_rn(vals[diag_l[k]], -c_l);
  }
  if (r >= 0) {
    vals[slot_rl[k]] = __dadd_rn(vals[slot_rl[k]], c_r);
    vals[diag_r[k]] = __dadd_rn(vals[diag_r[k]], -c_r);
  }
  if (u_face) {
    // src::div(u): rhs_ -= dot(u_f, Sf_out) for both cells (Source.cpp:11-15)
    const double ux = u_face[2 * f], uy = u_face[2 * f + 1];
    const double dl = __dadd_rn(__dmul_rn(ux, sfl_x[k]), __dmul_rn(uy, sfl_y[k]));
    const double dr = __dadd_rn(__dmul_rn(ux, sfr_x[k]), __dmul_rn(uy, sfr_y[k]));
    if (l >= 0) rhs[l] = __dadd_rn(rhs[l], -dl);
    if (r >= 0) rhs[r] = __dadd_rn(rhs[r], -dr);
  }
}

// Boundary colours: FIXED faces add -coeff to the owner's diagonal and
// coeff * phi_b to its rhs (Laplacian.h:66-69, 150-153); every boundary face
// contributes its flux to src::div.
__global__ void k_assemble_boundary(
    int nf, int off, const int32_t *__restrict__ cface,
    const int32_t *__restrict__ cl, const int32_t *__restrict__ bc,
    const double *__restrict__ dot_l, const double *__restrict__ msq,
    const int32_t *__restrict__ diag_l, const double *__restrict__ sfl_x,
    const double *__restrict__ sfl_y, const double *__restrict__ gamma_face,
    double gamma_scalar, const double *__restrict__ bc_value,
    const double *__restrict__ u_face, double *__restrict__ vals,
    double *__restrict__ rhs) {
  const int k = off + blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= off + nf) return;
  const int f = cface[k];
  const int l = cl[k];
  if (l < 0) return;  // owner is not a fluid row (ghost-cell IB equations)
  double acc = rhs[l];
  if (bc[k] == PG_BC_FIXED) {
    const double g = gamma_face ? gamma_face[f] : gamma_scalar;
    const double c = __ddiv_rn(__dmul_rn(g, dot_l[k]), msq[k]);
    vals[diag_l[k]] = __dadd_rn(vals[diag_l[k]], -c);
    acc = __dadd_rn(acc, __dmul_rn(c, bc_value[f]));
  }
  if (u_face) {
    const double ux = u_face[2 * f], uy = u_face[2 * f + 1];
    acc = __dadd_rn(acc, -__dadd_rn(__dmul_rn(ux, sfl_x[k]), __dmul_rn(uy, sfl_y[k])));
  }
  rhs[l] = acc;
}

// ---------------------------------------------------- momentum operator
// ddt + div - laplacian of the vector equation (TimeDerivative.h:38-48,
// Divergence.h:8-53, Laplacian.h:7-47), coefficients shared by the x and y
// components, rhs[2n] (x then y).  fv::ddt first: diagonal V/dt, source
// -V u0/dt; the face colours then add the upwind fluxes and subtract the
// diffusion terms.
__global__ void k_momentum_init(int n, const int32_t *__restrict__ diag,
                                const double *__restrict__ vol, double dt,
                                const double *__restrict__ u0,
                                double *__restrict__ vals,
                                double *__restrict__ rhs) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  const double v = vol[c];
  vals[diag[c]] = v / dt;
  rhs[c] = -v * u0[2 * c] / dt;
  rhs[n + c] = -v * u0[2 * c + 1] / dt;
}

__global__ void k_momentum_interior(
    int nf, int off, const int32_t *__restrict__ cface,
    const int32_t *__restrict__ cl, const int32_t *__restrict__ cr,
    const double *__restrict__ dot_l, const double *__restrict__ dot_r,
    const double *__restrict__ msq, const int32_t *__restrict__ slot_lr,
    const int32_t *__restrict__ slot_rl, const int32_t *__restrict__ diag_l,
    const int32_t *__restrict__ diag_r, const double *__restrict__ sfl_x,
    const double *__restrict__ sfl_y, const double *__restrict__ sfr_x,
    const double *__restrict__ sfr_y, double nu, double theta,
    const double *__restrict__ u0, const double *__restrict__ uf, int n,
    double *__restrict__ vals, double *__restrict__ rhs) {
  const int k = off + blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= off + nf) return;
  const int f = cface[k], l = cl[k], r = cr[k];
  const double ux = uf[2 * f], uy = uf[2 * f + 1];
  const double m2 = msq[k];
  // per side: flux F = u_f . Sf_out, diffusion coefficient c
  const double Fl = ux * sfl_x[k] + uy * sfl_y[k];
  const double Fr = ux * sfr_x[k] + uy * sfr_y[k];
  const double cll = nu * dot_l[k] / m2, crr = nu * dot_r[k] / m2;
  const double om = 1. - theta;
  vals[diag_l[k]] += theta * fmax(Fl, 0.) + theta * cll;
  vals[slot_lr[k]] += theta * fmin(Fl, 0.) - theta * cll;
  vals[diag_r[k]] += theta * fmax(Fr, 0.) + theta * crr;
  vals[slot_rl[k]] += theta * fmin(Fr, 0.) - theta * crr;
  if (om != 0.) {
    for (int d = 0; d < 2; ++d) {
      const double ul = u0[2 * l + d], ur = u0[2 * r + d];
      rhs[d * n + l] += om * (fmax(Fl, 0.) * ul + fmin(Fl, 0.) * ur) - om * cll * (ur - ul);
      rhs[d * n + r] += om * (fmax(Fr, 0.) * ur + fmin(Fr, 0.) * ul) - om * crr * (ul - ur);
    }
  }
}

__global__ void k_momentum_boundary(
    int nf, int off, const int32_t *__restrict__ cface,
    const int32_t *__restrict__ cl, const int32_t *__restrict__ bc,
    const double *__restrict__ dot_l, const double *__restrict__ msq,
    const int32_t *__restrict__ diag_l, const double *__restrict__ sfl_x,
    const double *__restrict__ sfl_y, double nu, double theta,
    const double *__restrict__ u0, const double *__restrict__ uf, int n,
    double *__restrict__ vals, double *__restrict__ rhs) {
  const int k = off + blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= off + nf) return;
  const int f = cface[k], l = cl[k];
  const double ux = uf[2 * f], uy = uf[2 * f + 1];
  const double F = ux * sfl_x[k] + uy * sfl_y[k];
  const double om = 1. - theta;
  if (bc[k] == PG_BC_FIXED) {
    const double c = nu * dot_l[k] / msq[k];
    vals[diag_l[k]] += theta * c;
    for (int d = 0; d < 2; ++d) {
      const double ub = uf[2 * f + d];
      rhs[d * n + l] += theta * F * ub + om * F * ub;            // div
      rhs[d * n + l] -= theta * c * ub + om * c * (ub - u0[2 * l + d]);  // -lap
    }
  } else if (bc[k] == PG_BC_NORMAL_GRADIENT) {
    vals[diag_l[k]] += theta * F;
    for (int d = 0; d < 2; ++d) rhs[d * n + l] += om * F * u0[2 * l + d];
  }
}

// FiniteVolumeField::interpolateFaces(DISTANCE) + setBoundaryFaces for a
// normal-gradient field (FiniteVolumeField.tpp:130-183, Face.cpp:60-64)
// Face::distanceWeight (Face.cpp:54-58) of every interior face: with l1 =
// |x_f - x_r| and l2 = |x_f - x_l|, g = l1 / (l1 + l2) weights the lCell
// (FiniteVolumeField.tpp:130-162 interpolates g phi_l + (1 - g) phi_r).
// Geometry only: computed once per mesh; boundary faces get 1.
__global__ void k_face_weights(int nf, const int32_t *__restrict__ fl,
                               const int32_t *__restrict__ fr,
                               const double *__restrict__ fcx,
                               const double *__restrict__ fcy,
                               const double *__restrict__ cx,
                               const double *__restrict__ cy,
                               double *__restrict__ fw) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  const int l = fl[f], r = fr[f];
  if (r < 0) {
    fw[f] = 1.;
    return;
  }
  const double ax = __dadd_rn(fcx[f], -cx[r]), ay = __dadd_rn(fcy[f], -cy[r]);
  const double bx = __dadd_rn(fcx[f], -cx[l]), by = __dadd_rn(fcy[f], -cy[l]);
  const double l1 = __dsqrt_rn(__dadd_rn(__dmul_rn(ax, ax), __dmul_rn(ay, ay)));
  const double l2 = __dsqrt_rn(__dadd_rn(__dmul_rn(bx, bx), __dmul_rn(by, by)));
  fw[f] = __ddiv_rn(l1, __dadd_rn(l1, l2));
}

// g phi_l + (1 - g) phi_r on interior faces, phi_l on boundary faces
__device__ __forceinline__ double face_interp(int l, int r, double w,
                                              const double *__restrict__ cv) {
  if (r < 0) return cv[l];
  return __dadd_rn(__dmul_rn(w, cv[l]), __dmul_rn(__dadd_rn(1., -w), cv[r]));
}

__global__ void k_interp_faces(int nf, const int32_t *__restrict__ fl,
                               const int32_t *__restrict__ fr,
                               const double *__restrict__ fw,
                               const double *__restrict__ cv,
                               double *__restrict__ fv) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  fv[f] = face_interp(fl[f], fr[f], fw[f], cv);
}

// dt / rho_f (FractionalStepMultiphase.cpp:175-185 with the distance-weighted
// face interpolation FiniteVolumeField.tpp:130-162, Face.cpp:60-64)
__global__ void k_dt_over_rho(int nf, const int32_t *__restrict__ fl,
                              const int32_t *__restrict__ fr,
                              const double *__restrict__ fw,
                              const double *__restrict__ gc, double rho1,
                              double rho2, double dt, double *__restrict__ out) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  const double gf = face_interp(fl[f], fr[f], fw[f], gc);
  const double c = fmin(fmax(gf, 0.), 1.);
  const double rho = __dadd_rn(rho1, __dmul_rn(c, __dadd_rn(rho2, -rho1)));
  out[f] = __ddiv_rn(dt, rho);
}

// ScalarGradient::computeFaces (ScalarGradient.cpp:34-47)
__global__ void k_grad_faces(int nf, const int32_t *__restrict__ fl,
                             const int32_t *__restrict__ fr,
                             const double *__restrict__ fcx,
                             const double *__restrict__ fcy,
                             const double *__restrict__ cx,
                             const double *__restrict__ cy,
                             const double *__restrict__ phi,
                             const double *__restrict__ phi_face,
                             double *__restrict__ gf) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  const int l = fl[f], r = fr[f];
  double dx, dy, d;
  if (r >= 0) {
    dx = __dadd_rn(cx[r], -cx[l]);
    dy = __dadd_rn(cy[r], -cy[l]);
    d = __dadd_rn(phi[r], -phi[l]);
  } else {
    dx = __dadd_rn(fcx[f], -cx[l]);
    dy = __dadd_rn(fcy[f], -cy[l]);
    d = __dadd_rn(phi_face[f], -phi[l]);
  }
  const double m2 = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
  gf[2 * f] = __ddiv_rn(__dmul_rn(d, dx), m2);
  gf[2 * f + 1] = __ddiv_rn(__dmul_rn(d, dy), m2);
}

// ScalarGradient::compute(FACE_TO_CELL) (ScalarGradient.cpp:56-73): |Sf|
// weighted average of the face gradients over the links, in link order.
__global__ void k_grad_cells(int n, const int64_t *__restrict__ link_ptr,
                             const int32_t *__restrict__ link_face,
                             const double *__restrict__ fnx,
                             const double *__restrict__ fny,
                             const double *__restrict__ gf,
                             double *__restrict__ gc) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  double tx = 0., ty = 0., sx = 0., sy = 0.;
  for (int64_t k = link_ptr[c]; k < link_ptr[c + 1]; ++k) {
    const int f = link_face[k];
    const double ax = fabs(fnx[f]), ay = fabs(fny[f]);
    tx = __dadd_rn(tx, __dmul_rn(gf[2 * f], ax));
    ty = __dadd_rn(ty, __dmul_rn(gf[2 * f + 1], ay));
    sx = __dadd_rn(sx, ax);
    sy = __dadd_rn(sy, ay);
  }
  gc[2 * c] = __ddiv_rn(tx, sx);
  gc[2 * c + 1] = __ddiv_rn(ty, sy);
}

// --------------------------------------------------------- permutation
__global__ void k_permute_values(int nnz, const int32_t *__restrict__ psrc,
                                 const double *__restrict__ src,
                                 double *__restrict__ dst) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < nnz) dst[j] = src[psrc[j]];
}
// Repeated columns of a row are summed in the caller's order by one thread
// (they only occur in hand-built inputs, never in assembled equations).
__global__ void k_add_dups(int nd, const int32_t *__restrict__ dd,
                           const int32_t *__restrict__ ds,
                           const double *__restrict__ src,
                           double *__restrict__ dst) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  for (int k = 0; k < nd; ++k) dst[dd[k]] += src[ds[k]];
}
__global__ void k_permute_vec(int n, const int32_t *__restrict__ perm,
                              const double *__restrict__ src, double scale,
                              double *__restrict__ dst) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = scale * src[perm[i]];
}
__global__ void k_unpermute_vec(int n, const int32_t *__restrict__ perm,
                                const double *__restrict__ src,
                                double *__restrict__ dst) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[perm[i]] = src[i];
}

// Jacobi / identity preconditioner with the same fused updates.
template <class VT, class MT, int MODE>
__global__ void k_diag_apply(int n, const MT *__restrict__ dinv,
                             const VT *__restrict__ r, VT *__restrict__ pv,
                             const VT *__restrict__ v, VT *__restrict__ z,
                             const KScalars *__restrict__ sc) {
  if (sc && sc->done) return;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += gridDim.x * blockDim.x) {
    const VT x = pre_input<VT>(MODE, i, r, pv, v, sc);
    z[i] = dinv ? (VT)dinv[i] * x : x;
  }
}

__global__ void k_jacobi_diag(int n, const int32_t *__restrict__ prp,
                              const int32_t *__restrict__ pci,
                              const double *__restrict__ pv,
                              double *__restrict__ dinv) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double dv = 0.;
  for (int j = prp[i]; j < prp[i + 1]; ++j)
    if (pci[j] == i) dv = pv[j];
  dinv[i] = dv != 0. ? 1. / dv : 1.;
}

// ------------------------------------------------------ SpMV + Krylov
template <class VT, class MT>
__device__ __forceinline__ VT row_dot(const int32_t *__restrict__ rp,
                                      const int32_t *__restrict__ ci,
                                      const MT *__restrict__ val,
                                      const VT *__restrict__ x, int i) {
  VT s = 0;
  const int b = rp[i], e = rp[i + 1];
  for (int j = b; j < e; ++j) s += (VT)val[j] * x[ci[j]];
  return s;
}

// row i of the sliced ELLPACK copy: the 32 rows of a slice are one warp's
// (the block size is a multiple of 32), so each entry slot is one
// contiguous 256-byte value load and 128-byte column load; the padding adds
// 0 x x[i] after the row's entries, leaving the CSR sum unchanged
__device__ __forceinline__ double row_dot_sell(const SolverDev &d,
                                               const double *__restrict__ x,
                                               int i) {
  const int e0 = d.sell_ptr[i >> 5], w = (d.sell_ptr[(i >> 5) + 1] - e0) >> 5;
  const double *v = d.sell_val + e0 + (i & 31);
  const int32_t *c = d.sell_col + e0 + (i & 31);
  double s = 0.;
  for (int k = 0; k < w; ++k) s += v[32 * k] * x[c[32 * k]];
  return s;
}

template <class VT, class MT>
__device__ __forceinline__ VT row_dot_any(const SolverDev &d,
                                          const MT *__restrict__ val,
                                          const VT *__restrict__ x, int i) {
  if constexpr (std::is_same<VT, double>::value && std::is_same<MT, double>::value) {
    if (d.sell_val) return row_dot_sell(d, x, i);
  }
  return row_dot<VT, MT>(d.prp, d.pci, val, x, i);
}

// The BiCGStab recurrence after the x / r update (last block, thread 0):
// tot = {<rhat, r>, <r, r>}
__device__ __forceinline__ void update_scalars(KScalars *sc, const double (&tot)[2],
                                               double al, double om) {
  const double rho_new = tot[0];
  sc->rr = tot[1];
  sc->iter += 1;
  if (!finite(tot[0]) || !finite(tot[1])) {
    sc->status = PG_NON_FINITE;
    sc->done = 1;
  } else {
    // rho_prev/rho advance on every exit, so a residual replacement after
    // a stop can continue the recurrence
    if (om != 0. && sc->rho != 0.) sc->beta = (rho_new / sc->rho) * (al / om);
    sc->rho_prev = sc->rho;
    sc->rho = rho_new;
    if (tot[1] <= sc->tol2 * sc->bb) {
      sc->status = PG_OK;
      sc->done = 1;
    } else if (sc->iter >= sc->max_iter) {
      sc->status = PG_MAX_ITERS;
      sc->done = 1;
    } else if (rho_new == 0. || om == 0.) {
      sc->status = PG_BREAKDOWN;
      sc->done = 1;
    }
  }
}
// ... after the SpMV v = A phat: alpha from <rhat, v>
__device__ __forceinline__ void spmv_v_scalars(KScalars *sc, double rv) {
  sc->rv = rv;
  if (!finite(rv)) {
    sc->status = PG_NON_FINITE;
    sc->done = 1;
  } else if (rv == 0.) {
    sc->status = PG_BREAKDOWN;
    sc->done = 1;
  } else {
    sc->alpha = sc->rho / rv;
  }
}
// ... after the SpMV t = A shat: omega from <t, t> and <t, s>
__device__ __forceinline__ void spmv_t_scalars(KScalars *sc, const double (&tot)[2]) {
  sc->tt = tot[0];
  sc->ts = tot[1];
  sc->omega = tot[0] > 0. ? tot[1] / tot[0] : 0.;
}

template <class VT, class MT>
__global__ void __launch_bounds__(kVecBlock)
k_spmv_v(SolverDev d, const MT *__restrict__ val, const VT *__restrict__ ph,
         VT *__restrict__ v, const VT *__restrict__ rh, KScalars *sc,
         RedWork w) {
  pdl_wait();
  if (sc->done) return;
  double acc[1] = {0.};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < d.n;
       i += gridDim.x * blockDim.x) {
    const VT vi = row_dot_any<VT, MT>(d, val, ph, i);
    v[i] = vi;
    acc[0] += (double)rh[i] * (double)vi;
  }
  double tot[1];
  if (grid_reduce<1>(acc, w, tot) && threadIdx.x == 0) spmv_v_scalars(sc, tot[0]);
}

template <class VT, class MT>
__global__ void __launch_bounds__(kVecBlock)
k_spmv_t(SolverDev d, const MT *__restrict__ val, const VT *__restrict__ sh,
         VT *__restrict__ t, const VT *__restrict__ s, KScalars *sc,
         RedWork w) {
  pdl_wait();
  if (sc->done) return;
  double acc[2] = {0., 0.};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < d.n;
       i += gridDim.x * blockDim.x) {
    const VT ti = row_dot_any<VT, MT>(d, val, sh, i);
    t[i] = ti;
    acc[0] += (double)ti * (double)ti;
    acc[1] += (double)ti * (double)s[i];
  }
  double tot[2];
  if (grid_reduce<2>(acc, w, tot) && threadIdx.x == 0) spmv_t_scalars(sc, tot);
}

template <class VT>
__global__ void __launch_bounds__(kVecBlock)
k_update(int n, VT *__restrict__ x, VT *__restrict__ r,
         const VT *__restrict__ ph, const VT *__restrict__ sh,
         const VT *__restrict__ s, const VT *__restrict__ t,
         const VT *__restrict__ rh, KScalars *sc, RedWork w) {
  pdl_wait();
  if (sc->done) return;
  const double al = sc->alpha, om = sc->omega;
  const VT alv = (VT)al, omv = (VT)om;  // vector math in storage precision
  double acc[2] = {0., 0.};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += gridDim.x * blockDim.x) {
    x[i] = x[i] + alv * ph[i] + omv * sh[i];
    const VT ri = s[i] - omv * t[i];
    r[i] = ri;
    acc[0] += (double)rh[i] * (double)ri;
    acc[1] += (double)ri * (double)ri;
  }
  double tot[2];
  if (grid_reduce<2>(acc, w, tot) && threadIdx.x == 0)
    update_scalars(sc, tot, al, om);
}

// ---- streamed forms (the vectors and matrix tiles move through shared
// memory by bulk copies, tma.cuh; the same sums as the kernels above, each
// thread's in its tiles' order) ----
constexpr int kUpdStages = 4;   // tiles in flight per CTA, x / r update
constexpr int kSpmvStages = 3;  // tiles in flight per CTA, SpMV
constexpr int kSellMaxW = 16;   // widest slice the streamed SpMV takes

// x += alpha phat + omega shat; r = s - omega t; <rhat, r>, <r, r>
__global__ void __launch_bounds__(kTileN)
k_update_tma(int n, double *__restrict__ x, double *__restrict__ r,
             const double *__restrict__ ph, const double *__restrict__ sh,
             const double *__restrict__ s, const double *__restrict__ t,
             const double *__restrict__ rh, KScalars *sc, RedWork w) {
  extern __shared__ __align__(128) uint8_t smem[];
  __shared__ __align__(8) uint64_t bar[kUpdStages];
  pdl_wait();
  if (sc->done) return;
  const double al = sc->alpha, om = sc->omega;
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
  double acc[2] = {0., 0.};
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
      const double *stg = reinterpret_cast<const double *>(smem + b * kStage);
      double xv, pv, shv, sv, tv, rhv;
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
      x[i] = xv + al * pv + om * shv;
      const double ri = sv - om * tv;
      r[i] = ri;
      acc[0] += rhv * ri;
      acc[1] += ri * ri;
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
  if (grid_reduce<2>(acc, w, tot) && threadIdx.x == 0)
    update_scalars(sc, tot, al, om);
}

// SpMV on the sliced ELLPACK copy with its fused dot products:
// WHICH 0: out = v = A phat, <rhat, v> (dv = rhat); WHICH 1: out = t =
// A shat, <t, t>, <t, s> (dv = s).  A row's products are summed in its
// entry order, as row_dot_sell.
template <int WHICH>
__global__ void __launch_bounds__(kTileN)
k_spmv_tma(SolverDev d, const double *__restrict__ xin,
           double *__restrict__ out, const double *__restrict__ dv,
           KScalars *sc, RedWork w) {
  extern __shared__ __align__(128) uint8_t smem[];
  __shared__ __align__(8) uint64_t bar[kSpmvStages];
  pdl_wait();
  if (sc->done) return;
  const int tid = threadIdx.x, G = gridDim.x, blk = blockIdx.x;
  const int n = d.n, W = d.sell_w, ns = (n + 31) >> 5;
  const int n_tiles = (n + kTileN - 1) / kTileN;
  const int m = blk < n_tiles ? (n_tiles - 1 - blk) / G + 1 : 0;
  const size_t stage = sell_stage_bytes(W, 1);
  const void *const vsrc[1] = {dv};
  // entry range [a, b) of the k-th tile (thread 0, for the issue)
  auto range = [&](int k, int &a, int &b) {
    const int s0 = 8 * (blk + k * G);
    a = __ldg(d.sell_ptr + s0);
    b = __ldg(d.sell_ptr + (s0 + 8 < ns ? s0 + 8 : ns));
  };
  // this thread's slice of the k-th tile: the tile's first entry and the
  // slice's entry range
  auto slice_of = [&](int k, int &ta, int &lo, int &hi) {
    const int j = blk + k * G;
    const int i = j * kTileN + tid;
    ta = lo = hi = 0;
    if (i < n) {
      ta = __ldg(d.sell_ptr + 8 * j);
      lo = __ldg(d.sell_ptr + (i >> 5));
      hi = __ldg(d.sell_ptr + (i >> 5) + 1);
    }
  };
  if (tid == 0) {
    for (int b = 0; b < kSpmvStages; ++b) mbar_init(&bar[b], 1);
    for (int k = 0; k < kSpmvStages && k < m; ++k) {
      int a, b;
      range(k, a, b);
      issue_sell_tile<1>(smem + k * stage, W, d.sell_val, d.sell_col, a, b,
                         vsrc, n, blk + k * G, &bar[k]);
    }
  }
  int ta = 0, lo = 0, hi = 0;
  if (m > 0) slice_of(0, ta, lo, hi);
  __syncthreads();
  double acc[2] = {0., 0.};
  int k = 0;
  bool failed = false;
  for (; k < m; ++k) {
    const int b = k % kSpmvStages;
    // loads for the next issue and the next tile, in flight during this one
    int na = 0, nb = 0;
    if (tid == 0 && k + kSpmvStages < m) range(k + kSpmvStages, na, nb);
    const int cta = ta, clo = lo, chi = hi;
    if (k + 1 < m) slice_of(k + 1, ta, lo, hi);
    const bool ok = mbar_wait_bounded(&bar[b], w.err, (uint32_t)((k / kSpmvStages) & 1));
    if (__syncthreads_or(!ok)) {
      failed = true;
      break;
    }
    const int j = blk + k * G;
    const int i = j * kTileN + tid;
    if (i < n) {
      const uint8_t *stg = smem + b * stage;
      const double *vals = reinterpret_cast<const double *>(stg);
      const int32_t *cols = reinterpret_cast<const int32_t *>(stg + (size_t)kTileN * W * 8);
      const double *dvec = reinterpret_cast<const double *>(stg + (size_t)kTileN * W * 12);
      const int o = clo - cta + (tid & 31), wq = (chi - clo) >> 5;
      double a = 0.;
      if (wq <= 8) {
        int32_t cc[8];
        double xv[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) cc[q] = q < wq ? cols[o + 32 * q] : 0;
#pragma unroll
        for (int q = 0; q < 8; ++q) xv[q] = q < wq ? __ldg(xin + cc[q]) : 0.;
#pragma unroll
        for (int q = 0; q < 8; ++q)
          if (q < wq) a += vals[o + 32 * q] * xv[q];
      } else {
        for (int q = 0; q < wq; ++q) a += vals[o + 32 * q] * __ldg(xin + cols[o + 32 * q]);
      }
      out[i] = a;
      const double dvi = tid < tile_bulk_count(n, j) ? dvec[tid] : dv[i];
      if (WHICH == 0) {
        acc[0] += dvi * a;
      } else {
        acc[0] += a * a;
        acc[1] += a * dvi;
      }
    }
    __syncthreads();  // stage b is free
    if (tid == 0 && k + kSpmvStages < m) {
      fence_proxy_async();
      issue_sell_tile<1>(smem + b * stage, W, d.sell_val, d.sell_col, na, nb,
                         vsrc, n, blk + (k + kSpmvStages) * G, &bar[b]);
    }
  }
  if (failed && tid == 0)
    for (int k2 = k + 1; k2 < m && k2 < k + kSpmvStages; ++k2)
      mbar_wait_bounded(&bar[k2 % kSpmvStages], nullptr, (uint32_t)((k2 / kSpmvStages) & 1));
  if (WHICH == 0) {
    double a1[1] = {acc[0]}, tot[1];
    if (grid_reduce<1>(a1, w, tot) && threadIdx.x == 0) spmv_v_scalars(sc, tot[0]);
  } else {
    double tot[2];
    if (grid_reduce<2>(acc, w, tot) && threadIdx.x == 0) spmv_t_scalars(sc, tot);
  }
}

// Fresh start from the true residual in r: rhat = r, p = v = 0,
// rho = <r, r>, alpha = omega = 1.
__global__ void __launch_bounds__(kVecBlock)
k_init_from_r(int n, const double *__restrict__ r, double *__restrict__ rh,
              double *__restrict__ p, double *__restrict__ v, KScalars *sc,
              RedWork w) {
  double acc[1] = {0.};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += gridDim.x * blockDim.x) {
    const double ri = r[i];
    rh[i] = ri;
    p[i] = 0.;
    v[i] = 0.;
    acc[0] += ri * ri;
  }
  double tot[1];
  if (grid_reduce<1>(acc, w, tot) && threadIdx.x == 0) {
    sc->rr = tot[0];
    sc->rho = tot[0];
    sc->rho_prev = 1.;
    sc->alpha = 1.;
    sc->omega = 1.;
    sc->beta = tot[0];
    sc->status = PG_OK;
    sc->done = 0;
    if (!finite(tot[0]) || tot[0] == 0.) {
      sc->status = tot[0] == 0. ? PG_OK : PG_NON_FINITE;
      sc->done = 1;
    }
  }
}

// Residual replacement: r already holds b - A x; the search directions are
// kept and rho_{i+1}, beta_i are recomputed from the replaced r.
__global__ void __launch_bounds__(kVecBlock)
k_replace_r(int n, const double *__restrict__ r, const double *__restrict__ rh,
            KScalars *sc, RedWork w) {
  double acc[2] = {0., 0.};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += gridDim.x * blockDim.x) {
    const double ri = r[i];
    acc[0] += rh[i] * ri;
    acc[1] += ri * ri;
  }
  double tot[2];
  if (grid_reduce<2>(acc, w, tot) && threadIdx.x == 0) {
    sc->rr = tot[1];
    sc->done = 0;
    sc->status = PG_OK;
    if (!finite(tot[0]) || !finite(tot[1]) || tot[0] == 0. ||
        sc->omega == 0. || sc->rho_prev == 0.) {
      sc->status = PG_BREAKDOWN;
      sc->done = 1;
    } else {
      sc->beta = (tot[0] / sc->rho_prev) * (sc->alpha / sc->omega);
      sc->rho = tot[0];
    }
  }
}

__global__ void __launch_bounds__(kVecBlock)
k_true_residual(SolverDev d, const double *__restrict__ val,
                const double *__restrict__ b, const double *__restrict__ x,
                double *__restrict__ r, KScalars *sc, RedWork w) {
  double acc[1] = {0.};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < d.n;
       i += gridDim.x * blockDim.x) {
    const double ri = x ? b[i] - row_dot<double, double>(d.prp, d.pci, val, x, i)
                        : b[i];
    if (r) r[i] = ri;
    acc[0] += ri * ri;
  }
  double tot[1];
  if (grid_reduce<1>(acc, w, tot) && threadIdx.x == 0) sc->rr_true = tot[0];
}

inline int blocks_for(int n, int bs) { return (n + bs - 1) / bs; }

// u -= (dt / rho) * grad p per cell and per face (FractionalStep.cpp:109-117,
// FractionalStepMultiphase.cpp:165-173); rho NULL means 1 (single phase:
// u -= dt * grad p).  The coefficient is formed first, as the reference
// evaluates timeStep / rho_(cell) * gradP_(cell).
__global__ void k_correct_velocity(int n, double dt,
                                   const double *__restrict__ rho,
                                   const double *__restrict__ grad,
                                   double *__restrict__ u) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += gridDim.x * blockDim.x) {
    const double c = rho ? __ddiv_rn(dt, rho[i]) : dt;
    u[2 * i] = __dadd_rn(u[2 * i], -__dmul_rn(c, grad[2 * i]));
    u[2 * i + 1] = __dadd_rn(u[2 * i + 1], -__dmul_rn(c, grad[2 * i + 1]));
  }
}

// FiniteVolumeField::setBoundaryFaces (FiniteVolumeField.tpp:165-183):
// normal-gradient and symmetry boundary faces take their cell's value,
// fixed ones keep theirs, interior faces are untouched
__global__ void k_set_boundary_faces(int nf, const int32_t *__restrict__ fl,
                                     const int32_t *__restrict__ fr,
                                     const int32_t *__restrict__ bc,
                                     const double *__restrict__ phi_cell,
                                     double *__restrict__ phi_face) {
  for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < nf;
       f += gridDim.x * blockDim.x)
    if (fr[f] < 0 && bc[f] != PG_BC_FIXED) phi_face[f] = phi_cell[fl[f]];
}

}  // namespace

// ---------------------------------------------------------------- launchers
void launch_assemble_interior(int nf, int off, const int32_t *cface,
                              const int32_t *cl, const int32_t *cr,
                              const double *dot_l, const double *dot_r,
                              const double *msq, const int32_t *slot_lr,
                              const int32_t *slot_rl, const int32_t *diag_l,
                              const int32_t *diag_r, const double *sfl_x,
                              const double *sfl_y, const double *sfr_x,
                              const double *sfr_y, const double *gamma_face,
                              double gamma_scalar, const double *u_face,
                              double *vals, double *rhs, cudaStream_t st) {
  if (nf <= 0) return;
  k_assemble_interior<<<blocks_for(nf, 256), 256, 0, st>>>(
      nf, off, cface, cl, cr, dot_l, dot_r, msq, slot_lr, slot_rl, diag_l,
      diag_r, sfl_x, sfl_y, sfr_x, sfr_y, gamma_face, gamma_scalar, u_face,
      vals, rhs);
  count_launches(1);
}

void launch_assemble_boundary(int nf, int off, const int32_t *cface,
                              const int32_t *cl, const int32_t *bc,
                              const double *dot_l, const double *msq,
                              const int32_t *diag_l, const double *sfl_x,
                              const double *sfl_y, const double *gamma_face,
                              double gamma_scalar, const double *bc_value,
                              const double *u_face, double *vals, double *rhs,
                              cudaStream_t st) {
  if (nf <= 0) return;
  k_assemble_boundary<<<blocks_for(nf, 256), 256, 0, st>>>(
      nf, off, cface, cl, bc, dot_l, msq, diag_l, sfl_x, sfl_y, gamma_face,
      gamma_scalar, bc_value, u_face, vals, rhs);
  count_launches(1);
}

void launch_correct_velocity(int n, double dt, const double *rho,
                             const double *grad, double *u, cudaStream_t st) {
  if (n <= 0) return;
  const int g = blocks_for(n, 256) < 2432 ? blocks_for(n, 256) : 2432;
  k_correct_velocity<<<g, 256, 0, st>>>(n, dt, rho, grad, u);
  count_launches(1);
}

void launch_set_boundary_faces(int nf, const int32_t *fl, const int32_t *fr,
                               const int32_t *bc, const double *phi_cell,
                               double *phi_face, cudaStream_t st) {
  if (nf <= 0) return;
  const int g = blocks_for(nf, 256) < 2432 ? blocks_for(nf, 256) : 2432;
  k_set_boundary_faces<<<g, 256, 0, st>>>(nf, fl, fr, bc, phi_cell, phi_face);
  count_launches(1);
}

void launch_momentum_init(int n, const int32_t *diag, const double *vol,
                          double dt, const double *u0, double *vals,
                          double *rhs, cudaStream_t st) {
  k_momentum_init<<<blocks_for(n, 256), 256, 0, st>>>(n, diag, vol, dt, u0,
                                                      vals, rhs);
  count_launches(1);
}
void launch_momentum_interior(int nf, int off, const int32_t *cface,
                              const int32_t *cl, const int32_t *cr,
                              const double *dot_l, const double *dot_r,
                              const double *msq, const int32_t *slot_lr,
                              const int32_t *slot_rl, const int32_t *diag_l,
                              const int32_t *diag_r, const double *sfl_x,
                              const double *sfl_y, const double *sfr_x,
                              const double *sfr_y, double nu, double theta,
                              const double *u0, const double *u_face, int n,
                              double *vals, double *rhs, cudaStream_t st) {
  if (nf <= 0) return;
  k_momentum_interior<<<blocks_for(nf, 256), 256, 0, st>>>(
      nf, off, cface, cl, cr, dot_l, dot_r, msq, slot_lr, slot_rl, diag_l,
      diag_r, sfl_x, sfl_y, sfr_x, sfr_y, nu, theta, u0, u_face, n, vals, rhs);
  count_launches(1);
}
void launch_momentum_boundary(int nf, int off, const int32_t *cface,
                              const int32_t *cl, const int32_t *bc,
                              const double *dot_l, const double *msq,
                              const int32_t *diag_l, const double *sfl_x,
                              const double *sfl_y, double nu, double theta,
                              const double *u0, const double *u_face, int n,
                              double *vals, double *rhs, cudaStream_t st) {
  if (nf <= 0) return;
  k_momentum_boundary<<<blocks_for(nf, 256), 256, 0, st>>>(
      nf, off, cface, cl, bc, dot_l, msq, diag_l, sfl_x, sfl_y, nu, theta, u0,
      u_face, n, vals, rhs);
  count_launches(1);
}
void launch_face_weights(int nf, const int32_t *fl, const int32_t *fr,
                         const double *fcx, const double *fcy,
                         const double *cx, const double *cy, double *fw,
                         cudaStream_t st) {
  if (nf <= 0) return;
  k_face_weights<<<blocks_for(nf, 256), 256, 0, st>>>(nf, fl, fr, fcx, fcy, cx,
                                                      cy, fw);
  count_launches(1);
}

void launch_interp_faces(int nf, const int32_t *fl, const int32_t *fr,
                         const double *fw, const double *cell_vals,
                         double *face_vals, cudaStream_t st) {
  if (nf <= 0) return;
  k_interp_faces<<<blocks_for(nf, 256), 256, 0, st>>>(nf, fl, fr, fw,
                                                      cell_vals, face_vals);
  count_launches(1);
}

void launch_dt_over_rho(int nf, const int32_t *fl, const int32_t *fr,
                        const double *fw, const double *gamma_cell,
                        double rho1, double rho2, double dt, double *out,
                        cudaStream_t st) {
  if (nf <= 0) return;
  k_dt_over_rho<<<blocks_for(nf, 256), 256, 0, st>>>(nf, fl, fr, fw,
                                                     gamma_cell, rho1, rho2,
                                                     dt, out);
  count_launches(1);
}

void launch_gradient(int n_cells, int nf, const int32_t *fl,
                     const int32_t *fr, const double *fcx, const double *fcy,
                     const double *cx, const double *cy,
                     const int64_t *link_ptr, const int32_t *link_face,
                     const int8_t *, const int8_t *, const double *fnx,
                     const double *fny, const double *phi,
                     const double *phi_face, double *grad_face,
                     double *grad_cell, cudaStream_t st) {
  k_grad_faces<<<blocks_for(nf, 256), 256, 0, st>>>(nf, fl, fr, fcx, fcy, cx,
                                                     cy, phi, phi_face,
                                                     grad_face);
  count_launches(1);
  if (grad_cell) {
    k_grad_cells<<<blocks_for(n_cells, 256), 256, 0, st>>>(
        n_cells, link_ptr, link_face, fnx, fny, grad_face, grad_cell);
    count_launches(1);
  }
}

__global__ void k_sell_values(int64_t n_ent, const int32_t *__restrict__ src,
                              const double *__restrict__ pvals,
                              double *__restrict__ out) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e < n_ent) out[e] = src[e] >= 0 ? pvals[src[e]] : 0.;
}

void launch_sell_values(int64_t n_ent, const int32_t *sell_src,
                        const double *pvals, double *sell_val, cudaStream_t st) {
  if (n_ent <= 0) return;
  k_sell_values<<<(int)((n_ent + 255) / 256), 256, 0, st>>>(n_ent, sell_src,
                                                            pvals, sell_val);
  count_launches(1);
}

void launch_permute_values(int nnz, const int32_t *psrc, const double *src,
                           double *dst, int n_dup, const int32_t *dup_dst,
                           const int32_t *dup_src, cudaStream_t st) {
  k_permute_values<<<blocks_for(nnz, 256), 256, 0, st>>>(nnz, psrc, src, dst);
  count_launches(1);
  if (n_dup > 0) {
    k_add_dups<<<1, 32, 0, st>>>(n_dup, dup_dst, dup_src, src, dst);
    count_launches(1);
  }
}

void launch_permute_vec(int n, const int32_t *perm, const double *src,
                        double scale, double *dst, cudaStream_t st) {
  k_permute_vec<<<blocks_for(n, 256), 256, 0, st>>>(n, perm, src, scale, dst);
  count_launches(1);
}

void launch_unpermute_vec(int n, const int32_t *perm, const double *src,
                          double *dst, cudaStream_t st) {
  k_unpermute_vec<<<blocks_for(n, 256), 256, 0, st>>>(n, perm, src, dst);
  count_launches(1);
}

// The streamed SpMV when the sliced copy is there, narrow enough and the
// vectors are 16-byte aligned (PG_STREAM=0 keeps the thread-per-row forms)
bool stream_enabled() {
  static const bool on = [] {
    const char *e = std::getenv("PG_STREAM");
    return !(e && e[0] == '0');
  }();
  return on;
}
template <int WHICH>
bool launch_spmv_tma(const SolverDev &d, const double *xin, double *out,
                     const double *dv, KScalars *sc, RedWork w, cudaStream_t st) {
  if (!stream_enabled() || !d.sell_val || d.sell_w < 1 || d.sell_w > kSellMaxW ||
      !aligned16(dv) || !aligned16(d.sell_val) || !aligned16(d.sell_col) || d.n < 1)
    return false;
  const size_t smem = kSpmvStages * sell_stage_bytes(d.sell_w, 1);
  static size_t attr = 0;
  if (attr < smem) {
    cudaFuncSetAttribute(k_spmv_tma<WHICH>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)smem);
    attr = smem;
  }
  const int g = stream_grid((const void *)k_spmv_tma<WHICH>, smem,
                            (d.n + kTileN - 1) / kTileN, w.grid);
  launch_pdl(k_spmv_tma<WHICH>, g, kTileN, smem, st, d, xin, out, dv, sc, w);
  count_launches(1);
  return true;
}

template <class VT, class MT>
void launch_spmv_v(const SolverDev &d, const MT *val, const VT *ph, VT *v,
                   const VT *rh, KScalars *sc, RedWork w, cudaStream_t st) {
  if constexpr (std::is_same<VT, double>::value && std::is_same<MT, double>::value)
    if (launch_spmv_tma<0>(d, ph, v, rh, sc, w, st)) return;
  launch_pdl(k_spmv_v<VT, MT>, w.grid, kVecBlock, 0, st, d, val, ph, v, rh, sc, w);
  count_launches(1);
}
template <class VT, class MT>
void launch_spmv_t(const SolverDev &d, const MT *val, const VT *sh, VT *t,
                   const VT *s, KScalars *sc, RedWork w, cudaStream_t st) {
  if constexpr (std::is_same<VT, double>::value && std::is_same<MT, double>::value)
    if (launch_spmv_tma<1>(d, sh, t, s, sc, w, st)) return;
  launch_pdl(k_spmv_t<VT, MT>, w.grid, kVecBlock, 0, st, d, val, sh, t, s, sc, w);
  count_launches(1);
}
template <class VT>
void launch_update(int n, VT *x, VT *r, const VT *ph, const VT *sh,
                   const VT *s, const VT *t, const VT *rh, KScalars *sc,
                   RedWork w, cudaStream_t st) {
  if constexpr (std::is_same<VT, double>::value) {
    if (stream_enabled() && n > 0 && aligned16(x) && aligned16(r) &&
        aligned16(ph) && aligned16(sh) && aligned16(s) && aligned16(t) &&
        aligned16(rh)) {
      constexpr size_t smem = kUpdStages * 6 * kTileN * 8;
      static bool attr = false;
      if (!attr) {
        cudaFuncSetAttribute(k_update_tma, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
        attr = true;
      }
      const int g = stream_grid((const void *)k_update_tma, smem,
                                (n + kTileN - 1) / kTileN, w.grid);
      launch_pdl(k_update_tma, g, kTileN, smem, st, n, x, r, ph, sh, s, t, rh, sc, w);
      count_launches(1);
      return;
    }
  }
  launch_pdl(k_update<VT>, w.grid, kVecBlock, 0, st, n, x, r, ph, sh, s, t, rh, sc, w);
  count_launches(1);
}
void launch_init_from_r(int n, double *r, double *rh, double *p, double *v,
                        KScalars *sc, RedWork w, cudaStream_t st) {
  k_init_from_r<<<w.grid, kVecBlock, 0, st>>>(n, r, rh, p, v, sc, w);
  count_launches(1);
}
void launch_replace_r(int n, const double *r, const double *rh, KScalars *sc,
                      RedWork w, cudaStream_t st) {
  k_replace_r<<<w.grid, kVecBlock, 0, st>>>(n, r, rh, sc, w);
  count_launches(1);
}

void launch_true_residual(const SolverDev &d, const double *val,
                          const double *b, const double *x, double *r,
                          KScalars *sc, RedWork w, cudaStream_t st) {
  k_true_residual<<<w.grid, kVecBlock, 0, st>>>(d, val, b, x, r, sc, w);
  count_launches(1);
}
void launch_jacobi_diag(const SolverDev &d, const double *pvals, double *dinv,
                        cudaStream_t st) {
  k_jacobi_diag<<<blocks_for(d.n, 256), 256, 0, st>>>(d.n, d.prp, d.pci, pvals,
                                                      dinv);
  count_launches(1);
}

template <class VT, class MT>
void launch_diag_apply(int mode, const SolverDev &d, const MT *dinv,
                       const VT *r, VT *pv, const VT *v, VT *z,
                       const KScalars *sc, cudaStream_t st) {
  const int g = blocks_for(d.n, 256) < 1216 ? blocks_for(d.n, 256) : 1216;
  if (mode == 0)
    k_diag_apply<VT, MT, 0><<<g, 256, 0, st>>>(d.n, dinv, r, pv, v, z, sc);
  else if (mode == 1)
    k_diag_apply<VT, MT, 1><<<g, 256, 0, st>>>(d.n, dinv, r, pv, v, z, sc);
  else
    k_diag_apply<VT, MT, 2><<<g, 256, 0, st>>>(d.n, dinv, r, pv, v, z, sc);
  count_launches(1);
}

#define PG_INST(VT, MT)                                                       \
  template void launch_diag_apply<VT, MT>(int, const SolverDev &, const MT *, \
                                          const VT *, VT *, const VT *, VT *, \
                                          const KScalars *, cudaStream_t);    \
  template void launch_spmv_v<VT, MT>(const SolverDev &, const MT *,          \
                                      const VT *, VT *, const VT *,           \
                                      KScalars *, RedWork, cudaStream_t);     \
  template void launch_spmv_t<VT, MT>(const SolverDev &, const MT *,          \
                                      const VT *, VT *, const VT *,           \
                                      KScalars *, RedWork, cudaStream_t);
PG_INST(double, double)
template void launch_update<double>(int, double *, double *, const double *,
                                    const double *, const double *,
                                    const double *, const double *,
                                    KScalars *, RedWork, cudaStream_t);

}  // namespace pg
