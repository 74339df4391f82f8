// Device kernels of libphase_gb300 (sm_103a).  Declarations shared by
// kernels.cu and the host drivers in capi.cu.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

struct pg_lu;

namespace pg {

// Host-side count of kernel launches issued by the library.
void count_launches(int k);
uint64_t launch_count();

// Programmatic dependent launch.  A kernel started by launch_pdl may be
// scheduled while the previous kernel of its stream is finishing (captured
// CUDA graphs keep this as a programmatic edge): it calls pdl_wait() before
// touching anything that kernel writes (the wait returns once that grid
// has completed and its writes are visible; at once without PDL).  The
// kernels leave the trigger for the next launch implicit (at exit): an
// explicit pdl_trigger() at a kernel's start measured 12 % slower solves on
// the 1M-row bubble, the next grid's waiting CTAs taking SM resources from
// the running one.  PG_PDL=0 in the environment launches them in plain
// stream order.
__device__ __forceinline__ void pdl_wait() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
}
__device__ __forceinline__ void pdl_trigger() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
bool pdl_enabled();
// streamed (bulk-copy) forms of the SpMVs and the x / r update
// (PG_STREAM=0 in the environment keeps the thread-per-row forms)
bool stream_enabled();
template <typename... KArgs, typename... Args>
inline void launch_pdl(void (*kern)(KArgs...), dim3 grid, dim3 block,
                       size_t smem, cudaStream_t st, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = pdl_enabled() ? 1 : 0;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, kern, args...);
}

// Scalars of one BiCGStab run, resident in device memory.  The last block of
// every reducing kernel updates them, so the iteration never waits on the
// host; kernels read them at entry and return at once when `done` is set.
struct KScalars {
  double rho, rho_prev, alpha, omega, beta;
  double rv, tt, ts, rr, bb;
  double rr_true;
  double tol2;
  // float-float copies of alpha, omega, beta for the mixed-precision
  // kernels, written next to the FP64 values by the same thread
  float2 alpha_dd, omega_dd, beta_dd;
  // batched solves: device-side reliable updates (batch.cu)
  double rr_ref;  // true ||r||^2 at the last replacement
  int action;     // 0 none, 1 confirm convergence, 2 restart, 3 replace
  int restarts;
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
  int grid;              // at least the grid of every kernel that reduces
  int *err = nullptr;    // set when a bounded device wait runs out
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
void launch_momentum_init(int n, const int32_t *diag, const double *vol,
                          double dt, const double *u0, double *vals,
                          double *rhs, cudaStream_t st);
void launch_momentum_interior(int nf, int off, const int32_t *cface,
                              const int32_t *cl, const int32_t *cr,
                              const double *dot_l, const double *dot_r,
                              const double *msq, const int32_t *slot_lr,
                              const int32_t *slot_rl, const int32_t *diag_l,
                              const int32_t *diag_r, const double *sfl_x,
                              const double *sfl_y, const double *sfr_x,
                              const double *sfr_y, double nu, double theta,
                              const double *u0, const double *u_face, int n,
                              double *vals, double *rhs, cudaStream_t st);
void launch_momentum_boundary(int nf, int off, const int32_t *cface,
                              const int32_t *cl, const int32_t *bc,
                              const double *dot_l, const double *msq,
                              const int32_t *diag_l, const double *sfl_x,
                              const double *sfl_y, double nu, double theta,
                              const double *u0, const double *u_face, int n,
                              double *vals, double *rhs, cudaStream_t st);
void launch_correct_velocity(int n, double dt, const double *rho,
                             const double *grad, double *u, cudaStream_t st);
void launch_set_boundary_faces(int nf, const int32_t *fl, const int32_t *fr,
                               const int32_t *bc, const double *phi_cell,
                               double *phi_face, cudaStream_t st);
// fw: Face::distanceWeight of every face (1 on boundary faces), made once
// per mesh by launch_face_weights
void launch_face_weights(int nf, const int32_t *fl, const int32_t *fr,
                         const double *fcx, const double *fcy,
                         const double *cx, const double *cy, double *fw,
                         cudaStream_t st);
void launch_interp_faces(int nf, const int32_t *fl, const int32_t *fr,
                         const double *fw, const double *cell_vals,
                         double *face_vals, cudaStream_t st);
void launch_dt_over_rho(int nf, const int32_t *fl, const int32_t *fr,
                        const double *fw, const double *gamma_cell,
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
//   uint16 lvl[nlev+2]   level boundaries (subdomain-local rows) + sentinel
//   uint16 cols[K][nr]   slot-major; K = KL + KU slots: L columns then U
//                        columns, 0xFFFF marks an unused slot
//   MT     vals[K+1][nr] slot-major L multipliers, U values, then 1/u_ii
struct SubMeta {
  int32_t r0, nr, nlev, K, KL, rec_off, col_off, val_off, rec_bytes,
      slot_base, pad0, pad1;
};
constexpr uint16_t kPadCol = 0xFFFF;

// Streaming form of a sweep group's factor for the apply kernel (a group is
// one subdomain, or two whose levels fit side by side in a warp): the
// levels' L data (ascending) and U data + 1/u_ii (descending) are cut into
// level-aligned pieces that TMA double-buffers through shared memory.
//   header: uint16 lev[nlev][4] = {a0, w0, a1, w1}: level l is group-local
//           rows [a0, a0+w0) of the first subdomain and [a1, a1+w1) of the
//           second (w1 = 0 for a single subdomain); lane t < w0 sweeps row
//           a0+t, lane w0 <= t < w0+w1 row a1+t-w0;
//           int32 nF, nB, int32 table[nF+nB][3] = {level, byte offset,
//           bytes} (forward pieces start at `level`; backward pieces start
//           at `level` and run downwards)
//   level blob (forward):  uint16 cols[KL][w] | MT vals[KL][w]
//   level blob (backward): uint16 cols[KU][w] | MT vals[KU][w] | MT dinv[w]
//   every array padded to 16 bytes; w = w0 + w1; columns are group-local;
//   an unused slot has column nr (the kernel keeps z[nr] = 0) and value 0
struct StreamMeta {
  int32_t r0, nr, nlev, KL, KU, rec_off, hdr_bytes, max_piece;
  // the first two pieces (offsets in the record), loaded at kernel start
  int32_t p0_off, p0_bytes, p1_off, p1_bytes;
  // the group's subdomains: sub0 .. sub0+nsub-1 (nsub 1 or 2), the first
  // holding group-local rows [0, nr0)
  int32_t sub0, nsub, nr0, pad0;
};

// Line form of a sweep group's factor, for subdomains that are rectangular
// blocks of a structured grid (5-point rows: the L part of row (i, j) holds
// at most (i-1, j) and (i, j-1), the U part (i+1, j) and (i, j+1), so row
// (i, j) is on level i + j).  Lane i of a member owns grid line i and walks
// it one row per level: the value of (i-1, j) comes from lane i-1 by a warp
// shuffle and that of (i, j-1) is the lane's own previous row, so no level
// waits for shared memory.  A pair group puts two blocks of at most 16
// lines side by side (member m uses lanes 16 m .. 16 m + 15); a single
// block may have up to 32 lines.  Two record layouts (a missing neighbour
// has weight 0 in both):
// * line-major, for FP32 weights (k_ilu0_apply_line): member m's row (i, j)
//   has position nr0 m + i len_m + j, and each lane reads its own line's
//   weights in order; map, forward and backward weights are all held in
//   shared memory
//     map:      uint16 map[nr]: the line-major position of the group's
//               level-order row r (padded to 16 bytes)
//     forward:  WT f[nr][2]  {weight of (i-1, j), of (i, j-1)} by position
//     backward: WT b[nr][3]  {weight of (i+1, j), of (i, j+1), 1/u_ii}
//     (each padded to 16 bytes: pieces p0 and p1, loaded at kernel start)
// * level-major, for 8-byte weights (k_ilu0_apply_line_lv), streamed in
//   pieces through two shared-memory buffers:
//     header: per level 8 bytes {uint16 a0, a1; uint8 w0, lo0, w1, lo1}:
//             member m's rows of level l are group-local rows a_m ..
//             a_m+w_m-1 on lines lo_m .. lo_m+w_m-1; then int32 nF, nB and
//             the piece table int32[nF+nB][3] = {level, byte offset, bytes}
//     level blob (forward):  MT f[w][2]  {weight of (i-1, j), of (i, j-1)}
//     level blob (backward): MT b[w][3]  {weight of (i+1, j), of (i, j+1),
//                                         1/u_ii}
//     entry t of a level: member 0's lines first (t = i - lo0), then member
//     1's (t = w0 + i - lo1); blobs padded to 16 bytes; w = w0 + w1.
struct LineMeta {
  int32_t r0, nr, nlev, rec_off, hdr_bytes, max_piece;
  int32_t p0_off, p0_bytes, p1_off, p1_bytes;  // forward, backward weights
  int32_t sub0, nsub, nr0, lanes;  // lanes per member: 16 (pair) or 32
  int32_t buf1;    // byte offset of piece buffer 1 from buffer 0
  int32_t zs_off;  // byte offset of the group's z vector (line-major) in
                   // shared memory
  int16_t lines0, lines1;  // line-major form: grid lines of member 0 / 1
  uint16_t len0, len1;     // line-major form: line length of member 0 / 1
};

// Step form of the factor for the float-float sweep of the mixed solver,
// used when every row has at most 3 L and 3 U entries (quadrilateral and
// triangle meshes).  A step is one warp-wide slice of a level (up to 32
// rows):
//   uint32 idx[32][4]  byte offsets into the subdomain's z vector (8-byte
//                      entries) of {row, c0, c1, c2}; unused: nr (z[nr] = 0)
//   float2 val[32][4]  {w0, w1, w2, 1/u_ii} as float pairs
// Forward steps (L parts, levels ascending) come first, then backward steps
// (U parts and 1/u_ii, levels descending); pieces are kStepsPerPiece steps.
struct StepMeta {
  int32_t r0, nr, n_fwd, n_bwd, rec_off, pad0, pad1, pad2;
};
constexpr int kStepsPerPiece = 8;
constexpr int kStepIdxBytes = 32 * 16;
constexpr int kStepBytesDd = kStepIdxBytes + 32 * 4 * 8;

struct SolverDev {
  int n, nnz, n_sub;
  // permuted CSR
  const int32_t *prp, *pci;
  // its sliced ELLPACK copy for the FP64 SpMVs (32-row slices,
  // column-major; sell_val refreshed with the values; NULL: the CSR is
  // used)
  const int32_t *sell_ptr = nullptr, *sell_col = nullptr;
  const double *sell_val = nullptr;
  int sell_w = 0;  // widest slice (entries per row)
  // ILU(0) records (FP64)
  const SubMeta *meta64;
  uint8_t *rec64;
  const int32_t *rec_src;
  size_t smem64, smem_dd;  // dynamic smem of the staged applies (0 = too big)
  int max_kl, max_ku;      // widest L / U part of any row
  // FP64 streaming records and the factor -> stream value map
  const StreamMeta *smeta64;
  int n_grp;  // stream records (sweep groups of one or two subdomains)
  uint8_t *srec64;
  const int32_t *pack_src, *pack_dst64;
  int n_pack;
  // float-float step stream of the mixed solver (when use_steps)
  int use_steps;
  const StepMeta *tmeta_dd;
  uint8_t *srec_dd;
  const int32_t *pack_src_dd, *pack_dst_dd;
  int n_pack_dd;
  // float-float copy of the FP64 streaming records (same layout, float
  // pairs in place of doubles) and whether the mixed solver sweeps it
  // instead of the step stream
  uint8_t *srec_dds;
  int dd_stream;
  int *err;               // set when a bounded device wait runs out
  // batched solves: system of every subdomain (NULL for one system); the
  // apply kernels then read the scalars sc[sub_sys[subdomain]]
  const int32_t *sub_sys;
  // two-level Schwarz: the streamed sweeps write the sum of each
  // subdomain's input here, as a float pair (NULL: no coarse correction)
  float2 *csum;
  // deflated coarse correction (mode 3 of the streamed sweep): the input
  // is already p - (A Z) y and the sweep writes z + y_s, y_s the coarse
  // value of the row's subdomain in the sweep's arithmetic (double or
  // float pairs)
  const void *def_y;
  // line form (every group a structured block; n_lgrp > 0): FP64 records,
  // their float-pair copy for the mixed solver, shared memory per CTA
  int n_lgrp;
  const LineMeta *lmeta;
  uint8_t *lrec64, *lrec_dds;
  size_t lsmem;
  const int32_t *lpack_src, *lpack_dst;
  int n_lpack;
  // FP32-weight line records of the mixed solver (mixed_sweep 3; n_lgrp32
  // > 0 when they are in use)
  int n_lgrp32;
  const LineMeta *lmeta32;
  uint8_t *lrec32;
  size_t lsmem32;
  const int32_t *lpack32_src, *lpack32_dst;
  int n_lpack32;
};



// Coarse space of the two-level Schwarz preconditioner (coarse.cu): the
// subdomain row ranges, the coupling structure of A_c = Z^T A Z, the dense
// K x K FP32 matrix (inverted in place by launch_coarse_setup), the
// original diagonal, the blocked Gauss-Jordan work arrays (pivot-block
// inverses 2 x 32 x 32, one per step parity; W 32 x K, V and C K x 32) and
// the subdomain sums of an application's input (float pairs).
struct CoarseDev {
  int K = 0, max_cnb = 0;
  const int32_t *sub_ptr = nullptr, *cptr = nullptr, *cnb = nullptr;
  const uint8_t *cslot = nullptr;
  float *ac = nullptr, *dg0 = nullptr;
  float *pinv = nullptr, *W = nullptr, *V = nullptr, *C = nullptr;
  float2 *csum = nullptr;
  // deflated application (cfg.coarse = 2): A Z per row, y, the deflated
  // input
  const int32_t *azp = nullptr, *azj = nullptr;
  const uint8_t *azslot = nullptr;
  double *azv = nullptr, *y = nullptr, *tmp = nullptr;
  // float-float copies for the mixed solver
  float2 *azv_dd = nullptr, *y_dd = nullptr, *tmp_dd = nullptr;
};
void launch_az_values(const CoarseDev &c, int n, const int32_t *prp,
                      const double *pvals, cudaStream_t st);
// pv = the preconditioner's input (fused update), csum = Z^T pv, y = A_c^-1 csum
void launch_def_pre(const CoarseDev &c, int mode, const double *r, double *pv,
                    const double *v, const KScalars *sc, cudaStream_t st);
// t = pv - (A Z) y
void launch_def_in(const CoarseDev &c, int n, const double *pv, double *t,
                   const KScalars *sc, cudaStream_t st);
// z += Z y
void launch_coarse_add(const CoarseDev &c, double *z, const KScalars *sc,
                       cudaStream_t st);
// the same in float-float (azv_dd, y_dd, tmp_dd)
void launch_def_pre_dd(const CoarseDev &c, int mode, const float2 *r,
                       float2 *pv, const float2 *v, const KScalars *sc,
                       cudaStream_t st);
void launch_def_in_dd(const CoarseDev &c, int n, const float2 *pv, float2 *t,
                      const KScalars *sc, cudaStream_t st);
void launch_coarse_add_dd(const CoarseDev &c, float2 *z, const KScalars *sc,
                          cudaStream_t st);

// Block-diagonal coarse space of a batch of independent systems: system t
// owns subdomains [k0[t], k0[t+1]) and a dense K_t x K_t FP32 block of A_c
// (then its inverse) at float offset off[t] of ac.
struct CoarseBatchDev {
  int n_sys = 0, max_cnb = 0, max_k = 0;
  const int32_t *k0 = nullptr;
  const int64_t *off = nullptr;
  const int32_t *sub_ptr = nullptr, *cptr = nullptr, *cnb = nullptr;
  const uint8_t *cslot = nullptr;
  const int32_t *sub_sys = nullptr;
  float *ac = nullptr;
  float2 *csum = nullptr;
  // deflated form (cfg.coarse = 2): A Z per row and y per subdomain
  const int32_t *azp = nullptr, *azj = nullptr;
  const double *azv = nullptr;
  double *y = nullptr;
};
// A_c blocks from the permuted values, each inverted in place (one CTA per
// system; n_blk = total floats of the blocks)
void launch_coarse_setup_b(const CoarseBatchDev &c, int K, int64_t n_blk,
                           const double *pvals, const int32_t *prp,
                           cudaStream_t st);
// deflated form for batches: pv = the input (fused update), y = A_t^-1
// Z^T pv per system, tmp = pv - A Z y; then (after the sweep) z += Z y
void launch_def_pre_b(const CoarseBatchDev &c, int K, int mode, const double *r,
                      double *pv, const double *v, double *tmp,
                      const KScalars *sc, cudaStream_t st);
void launch_coarse_add_b(const CoarseBatchDev &c, int K, double *z,
                         const KScalars *sc, cudaStream_t st);
// z += Z A_c^-1 Z^T in for the systems still running
void launch_coarse_apply_b(const CoarseBatchDev &c, int K, const double *in,
                           double *z, bool have_sums, const KScalars *sc,
                           cudaStream_t st);

// A_c from the permuted values, then A_c^-1 in place (the K elimination
// steps are captured into *gj_graph on first use when gj_graph is given)
// The coarse matrix assembled as a CSR in FP64 (cvals, the pattern of
// cptr / cnb) and inverted through the sparse LU into c.ac (FP32, dense)
int launch_coarse_setup_lu(const CoarseDev &c, pg_lu *lu,
                           double *cvals, const double *pvals,
                           const int32_t *prp, cudaGraphExec_t *graph,
                           cudaStream_t st);
void launch_coarse_setup(const CoarseDev &c, const double *pvals,
                         const int32_t *prp, cudaGraphExec_t *gj_graph,
                         cudaStream_t st);
// z += Z A_c^-1 Z^T in  (in and z in the permuted order); have_sums: the
// sweep already wrote Z^T in to c.csum (the streamed ILU(0) kernels do)
// (sc: the solve's scalars; the kernels do nothing once it has converged)
void launch_coarse_apply(const CoarseDev &c, const double *in, double *z,
                         bool have_sums, const KScalars *sc, cudaStream_t st);
void launch_coarse_apply_dd(const CoarseDev &c, const float2 *in, float2 *z,
                            bool have_sums, const KScalars *sc,
                            cudaStream_t st);

// sliced ELLPACK values from the permuted CSR values (0 on padding)
void launch_sell_values(int64_t n_ent, const int32_t *sell_src,
                        const double *pvals, double *sell_val, cudaStream_t st);
void launch_permute_values(int nnz, const int32_t *psrc, const double *src,
                           double *dst, int n_dup, const int32_t *dup_dst,
                           const int32_t *dup_src, cudaStream_t st);
void launch_permute_vec(int n, const int32_t *perm, const double *src,
                        double scale, double *dst, cudaStream_t st);
void launch_unpermute_vec(int n, const int32_t *perm, const double *src,
                          double *dst, cudaStream_t st);

// ILU(0) numeric factorisation into the FP64 factor records, then packed
// into the FP64 streaming records and, when to_dd, the float-float step
// stream; bad counts zero or non-finite pivots.
void launch_ilu0_factor(const SolverDev &d, const double *pvals, int *bad,
                        bool to_dd, cudaStream_t st);

// Preconditioner application with fused vector update.
//   mode 0: z = M^-1 in
//   mode 1: p = r + beta (p - omega v); z = M^-1 p   (p written back)
//   mode 2: s = r - alpha v;            z = M^-1 s   (s written back)
//   mode 3: z = B in + Z y, in = p - (A Z) y already formed by k_def_in
//           (the output half of the deflated coarse correction; streamed
//           sweep forms only)
// Mode 3 of the streamed ILU(0) sweep (d.def_y set); false when the
// streamed form is not available
bool launch_ilu0_apply_def(const SolverDev &d, const double *in, double *z,
                           const KScalars *sc, cudaStream_t st);
bool launch_ilu0_apply_def_dd(const SolverDev &d, const float2 *in, float2 *z,
                              const KScalars *sc, cudaStream_t st);

template <class VT, class MT>
void launch_precond(int precond, int mode, const SolverDev &d,
                    const MT *jdinv, const VT *r, VT *pv, const VT *v, VT *z,
                    const KScalars *sc, cudaStream_t st);

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
// Reliable updates (van der Vorst & Ye): restart the iteration from the
// true residual held in r (fresh shadow residual), or keep the search
// directions and only recompute rho/beta from the replaced r.
void launch_init_from_r(int n, double *r, double *rh, double *p, double *v,
                        KScalars *sc, RedWork w, cudaStream_t st);
void launch_replace_r(int n, const double *r, const double *rh, KScalars *sc,
                      RedWork w, cudaStream_t st);

// ---- mixed-precision (float-float) solver kernels, dd.cu / ilu.cu ----
// Vectors are float2 {hi, lo} in the permuted order; the matrix values are
// a float-float copy of the permuted FP64 values.  Dot products leave the
// kernels as FP64 scalars in KScalars, like the FP64 kernels'.
void launch_dd_split(int64_t n, const double *src, double scale, float2 *dst,
                     cudaStream_t st);
void launch_dd_join(int n, const float2 *src, double scale, double *dst,
                    cudaStream_t st);
// x64 += xw / scale; xw = 0
void launch_dd_fold(int n, double *x64, float2 *xw, double inv_scale,
                    cudaStream_t st);
// r = dd(r64 * scale); restart (rhat = r, p = v = 0, rho = <r,r>) when
// restart, else residual replacement (rho, beta from the new r)
void launch_dd_set_r(int n, const double *r64, double scale, float2 *r,
                     float2 *rh, float2 *p, float2 *v, bool restart,
                     KScalars *sc, RedWork w, cudaStream_t st);
void launch_dd_spmv_v(const SolverDev &d, const float2 *val, const float2 *ph,
                      float2 *v, const float2 *rh, KScalars *sc, RedWork w,
                      cudaStream_t st);
void launch_dd_spmv_t(const SolverDev &d, const float2 *val, const float2 *sh,
                      float2 *t, const float2 *s, KScalars *sc, RedWork w,
                      cudaStream_t st);
void launch_dd_update(int n, float2 *x, float2 *r, const float2 *ph,
                      const float2 *sh, const float2 *s, const float2 *t,
                      const float2 *rh, KScalars *sc, RedWork w,
                      cudaStream_t st);
// Jacobi / identity preconditioner on float pairs (dinv NULL: identity)
void launch_dd_diag_apply(int mode, int n, const float2 *dinv, const float2 *r,
                          float2 *pv, const float2 *v, float2 *z,
                          const KScalars *sc, cudaStream_t st);
// ILU(0) sweeps in float-float arithmetic over the step stream (ilu.cu)
void launch_ilu0_apply_dd(int mode, const SolverDev &d, const float2 *r,
                          float2 *pv, const float2 *v, float2 *z,
                          const KScalars *sc, cudaStream_t st);

// ---- batched solves (batch.cu) ----
// Tiles of rows: tile t covers permuted rows [tile_r0[t], tile_r1[t]) of
// system tile_sys[t]; the tiles of system s are [tile_ptr[s], tile_ptr[s+1]).
struct BatchTiles {
  const int32_t *tile_sys, *tile_r0, *tile_r1, *tile_ptr;
  int n_tiles;
};
// per-tile partial sums [kMaxDots][n_tiles] and one ticket per system
struct BatchRed {
  double *partials;
  unsigned int *tickets;
  int n_tiles;
};
void launch_b_init(const BatchTiles &T, const BatchRed &R, int block,
                   const int32_t *rp, const int32_t *ci, const double *val,
                   const double *b, const double *x, double *r, double *rh,
                   double *p, double *v, KScalars *sc, const int *init,
                   cudaStream_t st);
void launch_b_spmv_v(const BatchTiles &T, const BatchRed &R, int block,
                     const SolverDev &d, const double *val,
                     const double *ph, double *v, const double *rh,
                     KScalars *sc, cudaStream_t st);
void launch_b_spmv_t(const BatchTiles &T, const BatchRed &R, int block,
                     const SolverDev &d, const double *val,
                     const double *sh, double *t, const double *s,
                     KScalars *sc, cudaStream_t st);
void launch_b_update(const BatchTiles &T, const BatchRed &R, int block,
                     double *x, double *r, const double *ph, const double *sh,
                     const double *s, const double *t, const double *rh,
                     KScalars *sc, cudaStream_t st);
void launch_b_true_residual(const BatchTiles &T, const BatchRed &R, int block,
                            const int32_t *rp, const int32_t *ci,
                            const double *val, const double *b,
                            const double *x, double *r, const double *rh,
                            KScalars *sc, const int *sel, cudaStream_t st);
// end-of-chunk fix-up of the systems with a pending action: r = b - A x in
// FP64, then confirm convergence, replace the recursive residual, or
// restart with a fresh shadow residual
void launch_b_fix(const BatchTiles &T, const BatchRed &R, int block,
                  const int32_t *rp, const int32_t *ci, const double *val,
                  const double *b, const double *x, double *r, double *rh,
                  double *p, double *v, KScalars *sc, cudaStream_t st);
void launch_b_check(int n_sys, const KScalars *sc, int *chunks,
                    int max_chunks, cudaGraphConditionalHandle h,
                    cudaStream_t st);

// ---- TFQMR / GMRES drivers (krylov.cu) ----
// y = A x on the permuted CSR (FP64)
void launch_spmv_plain(const SolverDev &d, const double *val, const double *x,
                       double *y, cudaStream_t st);
// out = a x + b y (out may be x or y; b == 0 ignores y)
void launch_lincomb(int n, double a, const double *x, double b,
                    const double *y, double *out, cudaStream_t st);
// out[k] = <V_k, w> for the kn vectors V_k = V + k ld (partial: kn x 64
// scratch), reduced in a fixed order
void launch_mdot(int n, int kn, const double *V, size_t ld, const double *w,
                 double *partial, double *out, cudaStream_t st);
// w -= sum_k h[k] V_k
void launch_vsub(int n, int kn, const double *V, size_t ld, const double *h,
                 double *w, cudaStream_t st);

// rr_true = ||b - A x||^2 (FP64 matrix and vectors); x == NULL gives ||b||^2
void launch_true_residual(const SolverDev &d, const double *val,
                          const double *b, const double *x, double *r,
                          KScalars *sc, RedWork w, cudaStream_t st);

void launch_jacobi_diag(const SolverDev &d, const double *pvals, double *dinv,
                        cudaStream_t st);

// ILU(0) application (ilu.cu) for one fused-update mode, and the
// Jacobi/identity version (kernels.cu).
template <class VT, class MT>
void launch_ilu0_apply(int mode, const SolverDev &d, const VT *r, VT *pv,
                       const VT *v, VT *z, const KScalars *sc,
                       cudaStream_t st);
template <class VT, class MT>
void launch_diag_apply(int mode, const SolverDev &d, const MT *dinv,
                       const VT *r, VT *pv, const VT *v, VT *z,
                       const KScalars *sc, cudaStream_t st);

// Input of a preconditioner application with the fused BiCGStab update:
//   mode 0: z = M^-1 pv
//   mode 1: p = r + beta (p - omega v), written back to pv
//   mode 2: s = r - alpha v,            written to pv
// pre_combine: the same arithmetic on operands already loaded (ri = r[i],
// pi = pv[i], vi = v[i]; unused ones are ignored).
template <class VT>
__device__ __forceinline__ VT pre_combine(int mode, VT ri, VT pi, VT vi,
                                          const KScalars *sc) {
  // vector arithmetic in the storage precision; the scalars come from the
  // FP64 recurrences
  if (mode == 1) return ri + (VT)sc->beta * (pi - (VT)sc->omega * vi);
  if (mode == 2) return ri - (VT)sc->alpha * vi;
  return pi;
}

template <class VT>
__device__ __forceinline__ VT pre_input(int mode, int i, const VT *r, VT *pv,
                                        const VT *v, const KScalars *sc) {
  const VT zero = VT(0);
  const VT val = pre_combine<VT>(mode, mode ? r[i] : zero,
                                 mode != 2 ? pv[i] : zero,
                                 mode ? v[i] : zero, sc);
  if (mode) pv[i] = val;
  return val;
}

}  // namespace pg
