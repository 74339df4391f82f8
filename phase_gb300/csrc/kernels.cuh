// Device kernels of libphase_gb300 (sm_103a).  Declarations shared by
// kernels.cu and the host drivers in capi.cu.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

namespace pg {

// Host-side count of kernel launches issued by the library.
void count_launches(int k);
uint64_t launch_count();

// Scalars of one BiCGStab run, resident in device memory.  The last block of
// every reducing kernel updates them, so the iteration never waits on the
// host; kernels read them at entry and return at once when `done` is set.
struct KScalars {
  double rho, alpha, omega, beta;
  double rv, tt, ts, rr, bb;
  double rr_true;
  double tol2;
  int iter, max_iter;
  int done;    // 0 running, 1 stopped
  int status;  // PG_OK (converged candidate), PG_MAX_ITERS, PG_BREAKDOWN,
               // PG_NON_FINITE
};

constexpr int kVecBlock = 256;   // threads per block of vector/SpMV kernels
constexpr int kMaxDots = 3;      // fused dot products per kernel

// Reduction workspace: per-block partial sums and a completion ticket.
struct RedWork {
  double *partials;      // [kMaxDots][grid]
  unsigned int *ticket;  // one counter
  int grid;
};

// ---- assembly / field kernels (FP64, reference arithmetic) ----
void launch_assemble_interior(int nf, int off, const int32_t *cface,
                              const int32_t *cl, const int32_t *cr,
                              const double *dot_l, const double *dot_r,
                              const double *msq, const int32_t *slot_lr,
                              const int32_t *slot_rl, const int32_t *diag_l,
                              const int32_t *diag_r, const double *sfl_x,
                              const double *sfl_y, const double *sfr_x,
                              const double *sfr_y, const double *gamma_face,
                              double gamma_scalar, const double *u_face,
                              double *vals, double *rhs, cudaStream_t st);
void launch_assemble_boundary(int nf, int off, const int32_t *cface,
                              const int32_t *cl, const int32_t *bc,
                              const double *dot_l, const double *msq,
                              const int32_t *diag_l, const double *sfl_x,
                              const double *sfl_y, const double *gamma_face,
                              double gamma_scalar, const double *bc_value,
                              const double *u_face, double *vals, double *rhs,
                              cudaStream_t st);
void launch_dt_over_rho(int nf, const int32_t *fl, const int32_t *fr,
                        const double *fcx, const double *fcy, const double *cx,
                        const double *cy, const double *gamma_cell,
                        double rho1, double rho2, double dt, double *out,
                        cudaStream_t st);
void launch_gradient(int n_cells, int nf, const int32_t *fl,
                     const int32_t *fr, const double *fcx, const double *fcy,
                     const double *cx, const double *cy,
                     const int64_t *link_ptr, const int32_t *link_face,
                     const int8_t *sgn_l, const int8_t *sgn_r,
                     const double *fnx, const double *fny, const double *phi,
                     const double *phi_face, double *grad_face,
                     double *grad_cell, cudaStream_t st);

// ---- solver kernels ----
// One Schwarz subdomain's ILU(0) factor is a packed record, 16-byte aligned
// so one cp.async.bulk moves it into shared memory:
//   uint16 lvl[nlev+1]   level boundaries (subdomain-local rows)
//   uint16 cols[nr][K]   K = KL + KU slots: L columns then U columns,
//                        0xFFFF marks an unused slot
//   MT     vals[nr][K+1] L multipliers, U values, 1/u_ii
struct SubMeta {
  int32_t r0, nr, nlev, K, KL, rec_off, col_off, val_off, rec_bytes,
      slot_base, pad0, pad1;
};
constexpr uint16_t kPadCol = 0xFFFF;

struct SolverDev {
  int n, nnz, n_sub;
  // permuted CSR
  const int32_t *prp, *pci;
  // ILU(0) records (FP64 and FP32 copies)
  const SubMeta *meta64, *meta32;
  uint8_t *rec64, *rec32;
  const int32_t *rec_src;
  size_t smem64, smem32;  // dynamic smem of the staged apply (0 = too big)
  int *err;               // set when a bounded device wait runs out
};

void launch_permute_values(int nnz, const int32_t *psrc, const double *src,
                           double *dst, int n_dup, const int32_t *dup_dst,
                           const int32_t *dup_src, cudaStream_t st);
void launch_permute_vec(int n, const int32_t *perm, const double *src,
                        double scale, double *dst, cudaStream_t st);
void launch_unpermute_vec(int n, const int32_t *perm, const double *src,
                          double *dst, cudaStream_t st);

// ILU(0) numeric factorisation into the FP64 records (and the FP32 copy
// when to_fp32); bad counts zero or non-finite pivots.
void launch_ilu0_factor(const SolverDev &d, const double *pvals, int *bad,
                        bool to_fp32, cudaStream_t st);

// Preconditioner application with fused vector update.
//   mode 0: z = M^-1 in
//   mode 1: p = r + beta (p - omega v); z = M^-1 p   (p written back)
//   mode 2: s = r - alpha v;            z = M^-1 s   (s written back)
template <class VT, class MT>
void launch_precond(int precond, int mode, const SolverDev &d,
                    const MT *jdinv, const VT *r, VT *pv, const VT *v, VT *z,
                    const KScalars *sc, cudaStream_t st);

template <class VT, class MT>
void launch_krylov_init(const SolverDev &d, const MT *val, const VT *b,
                        const VT *x, VT *r, VT *rh, VT *p, VT *v, KScalars *sc,
                        RedWork w, cudaStream_t st);
template <class VT, class MT>
void launch_spmv_v(const SolverDev &d, const MT *val, const VT *ph, VT *v,
                   const VT *rh, KScalars *sc, RedWork w, cudaStream_t st);
template <class VT, class MT>
void launch_spmv_t(const SolverDev &d, const MT *val, const VT *sh, VT *t,
                   const VT *s, KScalars *sc, RedWork w, cudaStream_t st);
template <class VT>
void launch_update(int n, VT *x, VT *r, const VT *ph, const VT *sh,
                   const VT *s, const VT *t, const VT *rh, KScalars *sc,
                   RedWork w, cudaStream_t st);
// rr_true = ||b - A x||^2 (FP64 matrix and vectors); x == NULL gives ||b||^2
void launch_true_residual(const SolverDev &d, const double *val,
                          const double *b, const double *x, double *r,
                          KScalars *sc, RedWork w, cudaStream_t st);

void launch_jacobi_diag(const SolverDev &d, const double *pvals, double *dinv,
                        cudaStream_t st);

}  // namespace pg
