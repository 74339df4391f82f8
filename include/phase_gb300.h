/*
 * phase_gb300 -- GB300 (sm_103a) pressure assembly + BiCGStab/ILU solve for
 * the Phase 2D unstructured finite-volume solver.
 *
 * C ABI: plain pointers and sizes, opaque handles, int status codes.  No C++
 * exceptions cross this boundary.  Host buffers are owned by the caller;
 * device buffers are owned by the library.  A handle is not thread-safe: one
 * host thread drives it at a time, as Phase's single-threaded ranks do.
 * All work of the library is issued on one CUDA stream (pg_stream()).
 *
 * Reference interfaces each entry point replaces are cited as file:line
 * within the obrienadam/Phase source tree.
 */
#ifndef PHASE_GB300_H
#define PHASE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define PG_OK 0
#define PG_MAX_ITERS 1   /* solve stopped at max iterations */
#define PG_BREAKDOWN 2   /* BiCGStab breakdown (rho or <t,t> = 0) or zero pivot */
#define PG_NON_FINITE 3  /* NaN/Inf in the inputs or the iteration */
#define PG_BAD_ARG 4     /* invalid argument / size / handle */
#define PG_TIMEOUT 5     /* a bounded device wait ran out */
#define PG_CUDA_ERROR 6  /* a CUDA runtime call failed */

/* where a pointer argument lives */
#define PG_HOST 0
#define PG_DEVICE 1

/* boundary types, FiniteVolumeField<T>::BoundaryType
 * (src/2D/Unstructured/FiniteVolume/Field/FiniteVolumeField.h) */
#define PG_BC_FIXED 0
#define PG_BC_NORMAL_GRADIENT 1
#define PG_BC_SYMMETRY 2

/* which fv::laplacian overload an equation is assembled by */
#define PG_GAMMA_SCALAR 0 /* fv::laplacian(Scalar, phi)   Laplacian.h:49-83  */
#define PG_GAMMA_FACE 1   /* fv::laplacian(field, phi)    Laplacian.h:132-167 */

/* preconditioners */
#define PG_PREC_NONE 0
#define PG_PREC_JACOBI 1
#define PG_PREC_ILU0 2 /* additive Schwarz (overlap 0) with ILU(0) blocks, as
                          Ifpack2 "schwarz" + "RILUK" level-of-fill 0
                          (TrilinosBelosSparseMatrixSolver.cpp:63-85) */

/* Krylov methods (the Belos solver names of TrilinosBelosSparseMatrixSolver
 * .cpp:59-60, key "solver") */
#define PG_KRYLOV_BICGSTAB 0 /* "BICGSTAB" (the default) */
#define PG_KRYLOV_TFQMR 1    /* "TFQMR" */
#define PG_KRYLOV_GMRES 2    /* "GMRES" (restarted, right preconditioned) */

/* arithmetic of the Krylov iteration */
#define PG_FP64 0
#define PG_MIXED 1 /* float-float (pairs of FP32, about 48 bits) Krylov
                      vectors, SpMV, ILU(0) sweeps and updates on the FP32
                      pipes, scalars in FP64; the recursive residual is
                      replaced by the FP64 true residual b - A x whenever it
                      has fallen 1e4-fold and at convergence, which is judged
                      on the FP64 true residual.  A solve whose true residual
                      stalls is finished by the FP64 solver from its iterate
                      (pg_solve_stats.fp64_iters). */

typedef struct pg_mesh pg_mesh;
typedef struct pg_eqn pg_eqn;
typedef struct pg_solver pg_solver;

/* Last error message of the calling thread (never NULL). */
const char *pg_last_error(void);

/* The CUDA stream (cudaStream_t) all library work is issued on. */
void *pg_stream(void);

/* Blocks until all library work issued so far has finished. */
int pg_synchronize(void);

/* ------------------------------------------------------------------------
 * Mesh.  Replaces FiniteVolumeGrid2D::init(nodes, cptr, cind, origin)
 * (src/2D/Unstructured/FiniteVolumeGrid2D/FiniteVolumeGrid2D.cpp:20-35),
 * createCell (:84-114) and the link set-up of init() (:396-450): faces are
 * numbered in cell order by node-pair de-duplication, the first cell that
 * meets a face is its lCell, links are kept in face-id order.
 * nodes_xy[2*n_nodes], cptr[n_cells+1], cind[cptr[n_cells]] (host).
 * ---------------------------------------------------------------------- */
int pg_mesh_create(const double *nodes_xy, int64_t n_nodes,
                   const int64_t *cptr, const int64_t *cind, int64_t n_cells,
                   pg_mesh **out);
int pg_mesh_destroy(pg_mesh *m);
int pg_mesh_sizes(const pg_mesh *m, int64_t *n_cells, int64_t *n_faces,
                  int64_t *n_interior, int64_t *n_boundary);
/* Face data (host copies), face-id order: owner/neighbour cells (rcell = -1
 * on boundary faces), centroid and normal (Face.cpp:9-18). Any may be NULL. */
int pg_mesh_faces(const pg_mesh *m, int32_t *lcell, int32_t *rcell,
                  double *fx, double *fy, double *nx, double *ny);
/* Cell centroids and volumes (Cell.cpp:8-29). Any may be NULL. */
int pg_mesh_cells(const pg_mesh *m, double *cx, double *cy, double *vol);

/* ------------------------------------------------------------------------
 * Pressure equation on the device.  A pg_eqn is a FiniteVolumeEquation<Scalar>
 * (src/2D/Unstructured/FiniteVolume/Equation/FiniteVolumeEquation.h:14-98)
 * whose CSR lives in HBM.  Its sparsity pattern is that of CrsEquation after
 * fv::laplacian (CrsEquation.cpp:9-14,113-131): placeholder slots dropped,
 * entries in order of first addCoeff.  bc_type[n_faces] (host) fixes the
 * boundary type of each boundary face for the life of the equation.
 * ---------------------------------------------------------------------- */
int pg_eqn_create(const pg_mesh *m, int gamma_kind, const int32_t *bc_type,
                  pg_eqn **out);
/* FiniteVolumeField::setBoundaryFaces (FiniteVolumeField.tpp:165-183):
 * on boundary faces of type PG_BC_NORMAL_GRADIENT or PG_BC_SYMMETRY,
 * phi_face[f] = phi_cell[lCell(f)]; fixed boundary faces and interior faces
 * keep their values.  bc_type[n_faces] (the field's boundary type per
 * face), phi_cell[n_cells], phi_face[n_faces] in ptr_kind memory. */
int pg_set_boundary_faces(const pg_mesh *m, const int32_t *bc_type,
                          const double *phi_cell, double *phi_face,
                          int ptr_kind);

/* Projection step after the pressure solve: u -= dt / rho * grad p on every
 * cell and every face (FractionalStep::correctVelocity,
 * src/2D/Unstructured/Solvers/FractionalStep.cpp:109-117, and its
 * multiphase form FractionalStepMultiphase.cpp:165-173).  rho_cell[n] and
 * rho_face[nf] are both given (multiphase) or both NULL (rho = 1).
 * grad_cell/u_cell hold x,y per cell (2n), grad_face/u_face per face (2nf),
 * e.g. from pg_gradient; u_cell and u_face are updated in place. */
int pg_correct_velocity(const pg_mesh *m, double dt, const double *rho_cell,
                        const double *rho_face, const double *grad_cell,
                        const double *grad_face, double *u_cell,
                        double *u_face, int ptr_kind);

/* Ghost-cell immersed-boundary pressure equation of FractionalStepGCIB
 * (src/2D/Unstructured/Solvers/FractionalStepGCIB.cpp:44-46):
 *   (fv::laplacian(gamma, p) + ib.bcs(p)) == src::div(u)
 * for circles[3k..3k+2] = (cx, cy, r), k < n_circles.  Cells whose centroid
 * is strictly inside a circle are IB cells when a face or node neighbour
 * is outside it, else solid (GhostCellImmersedBoundary::updateCells,
 * GhostCellImmersedBoundary.cpp:12-30); the Laplacian and the source run
 * over the fluid cells; IB rows carry the bilinear image-point stencils of
 * GhostCellImmersedBoundary::bcs (:32-74) for ib_bc PG_BC_FIXED or
 * PG_BC_NORMAL_GRADIENT with value ib_ref, solid rows the identity.  The
 * classes and the IB stencils (boundary point, image point, the cells of
 * the node nearest to it, the 4x4 inverse) are built on the device; the
 * host builds the pattern from them, and the device assembly
 * (pg_assemble_laplacian) fills the fluid rows.  The
 * sum is CrsEquation::operator+ (CrsEquation.cpp:185-229), which leaves out
 * entries that are exactly zero: the device matrix keeps their slots (with
 * value 0, the same operator), and pg_eqn_export drops them, so the
 * exported CSR is CrsEquation's.  Fails with PG_BAD_ARG when an image
 * point's nearest node does not have four cells or a stencil matrix is
 * singular. */
int pg_eqn_create_gcib(const pg_mesh *m, int gamma_kind, const int32_t *bc_type,
                       int n_circles, const double *circles, int ib_bc,
                       double ib_ref, pg_eqn **out);
/* Moves the bodies of a ghost-cell IB equation: circles[3k..3k+2] are the
 * new (cx, cy, r), ib_ref the new boundary value, as
 * GhostCellImmersedBoundary::updateCells after the bodies' Motion::update
 * (FractionalStepDFIB.cpp:29-31 does both every step; OscillatingMotion.cpp:
 * 12-24 is one motion).  Classes and stencils are rebuilt on the device.
 * When every cell keeps its class and every IB row its non-zero columns,
 * the new IB rows are written into the equation's constant rows on the
 * device and *pattern_changed = 0: the pattern, and a solver's analysis of
 * it, stay valid.  Otherwise the equation is rebuilt with the new pattern
 * (a new pattern: a solver given it re-analyses) and *pattern_changed = 1.
 * Either way the next pg_assemble_laplacian assembles the moved equation.
 * Fails with PG_BAD_ARG for an equation without an IB, or as
 * pg_eqn_create_gcib (the equation is then unchanged, except after a
 * failure of the rebuild itself, after which it must be destroyed). */
int pg_eqn_update_gcib(pg_eqn *e, int n_circles, const double *circles,
                       double ib_ref, int *pattern_changed);
/* Cell classes of a ghost-cell IB equation: 0 fluid, 1 IB, 2 solid (all 0
 * for other equations).  cls[n_rows]. */
int pg_eqn_cell_class(const pg_eqn *e, int32_t *cls);
int pg_eqn_destroy(pg_eqn *e);
int pg_eqn_sizes(const pg_eqn *e, int64_t *n_rows, int64_t *nnz);

/* fv::laplacian(gamma, p) == src::div(u) assembled on the device by the
 * face-coloured kernels.  Replaces Laplacian.h:49-83 (gamma_face == NULL,
 * scalar gamma) or :132-167 (gamma_face[n_faces]), Source.cpp:5-21
 * (u_face_xy[2*n_faces], NULL = no divergence source) and
 * CrsEquation::operator==(Vector) (CrsEquation.cpp:309-311).
 * bc_value[n_faces] holds phi on FIXED boundary faces (may be NULL when no
 * face is FIXED).  ptr_kind says where the arrays live. */
int pg_assemble_laplacian(pg_eqn *e, const double *gamma_face,
                          double gamma_scalar, const double *bc_value,
                          const double *u_face_xy, int ptr_kind);

/* The diagonal coefficient a_P of every row (0 for a row without one),
 * diag[n] in ptr_kind memory: for a momentum equation the a_P of the SIMPLE
 * coefficient d = V / a_P. */
int pg_eqn_diagonal(const pg_eqn *e, double *diag, int ptr_kind);

/* Device addresses of the equation's values (nnz) and rhs_ (n, or 2n for a
 * momentum equation); valid until the equation is destroyed. */
int pg_eqn_device_values(const pg_eqn *e, double **vals, double **rhs);

/* Copy the assembled CSR + rhs_ (the equation's own right-hand side; the
 * solver receives -rhs_, FiniteVolumeEquation.tpp:73) to host buffers.
 * row_ptr[n+1], col_ind[nnz], vals[nnz], rhs[n] with nnz from
 * pg_eqn_sizes; any may be NULL.  A ghost-cell IB equation exports the
 * entries of its last assembly that are not exactly zero (CrsEquation's
 * operator+), row_ptr[n] of them. */
int pg_eqn_export(const pg_eqn *e, int32_t *row_ptr, int32_t *col_ind,
                  double *vals, double *rhs);

/* Momentum operator of the vector equation, assembled on the device:
 *   fv::ddt(u, dt) + fv::div(u_face, u, theta) - fv::laplacian(nu, u, theta)
 * (TimeDerivative.h:38-48, Divergence.h:8-53, Laplacian.h:7-47) -- the
 * predictor whose diagonal a_P gives the SIMPLE coefficient d = V/a_P.  Both
 * velocity components share one N x N coefficient matrix (the reference
 * stacks them as rows 0..N-1 and N..2N-1 with equal coefficients,
 * VectorFiniteVolumeEquation.cpp:5-30); rows hold the diagonal first, then
 * the neighbours in link order.  Explicit zero coefficients are kept (the
 * reference's CrsEquation::operator+= drops them; the values agree).
 * bc_type[n_faces] (host) as for pg_eqn_create; the equation's rhs holds
 * 2*N values (x then y).  u_old_cell[2*N] (x,y per cell), u_face[2*n_faces]
 * (the face velocities of the fluxes; on FIXED faces the boundary values). */
int pg_eqn_create_momentum(const pg_mesh *m, const int32_t *bc_type,
                           pg_eqn **out);
int pg_assemble_momentum(pg_eqn *e, double dt, double nu, double theta,
                         const double *u_old_cell, const double *u_face,
                         int ptr_kind);

/* FiniteVolumeField::interpolateFaces(DISTANCE) followed by setBoundaryFaces
 * for a normal-gradient field (FiniteVolumeField.tpp:130-183, Face.cpp:60-64):
 * face value g*phi_l + (1-g)*phi_r with the distance weight g, boundary faces
 * take the owner cell's value.  cell_vals[n_cells] in, face_vals[n_faces]
 * out. */
int pg_interpolate_faces(const pg_mesh *m, const double *cell_vals,
                         double *face_vals, int ptr_kind);

/* Face coefficient timeStep / rho_f with rho_f = rho1 + clamp(gamma_f,0,1)
 * (rho2 - rho1) and gamma_f the distance-weighted face interpolation of the
 * cell volume fraction (FractionalStepMultiphase.cpp:175-185,
 * FiniteVolumeField.tpp:130-162, ScalarFiniteVolumeField.cpp:68-81).
 * Boundary faces take the owner cell's value (normal-gradient gamma).
 * gamma_cell[n_cells] in, coeff_face[n_faces] out. */
int pg_face_dt_over_rho(const pg_mesh *m, const double *gamma_cell,
                        double rho1, double rho2, double dt,
                        double *coeff_face, int ptr_kind);

/* ScalarGradient::computeFaces + compute(FACE_TO_CELL)
 * (src/2D/Unstructured/FiniteVolume/Field/ScalarGradient.cpp:34-74).
 * phi_cell[n_cells], phi_face[n_faces] (boundary values) in;
 * grad_face[2*n_faces], grad_cell[2*n_cells] out (either may be NULL). */
int pg_gradient(const pg_mesh *m, const double *phi_cell,
                const double *phi_face, double *grad_face, double *grad_cell,
                int ptr_kind);

/* ------------------------------------------------------------------------
 * Learned initial guess (no counterpart in the reference, which always
 * restarts BiCGStab from the previous solution): a 3-layer message-passing
 * network of width 32 on the matrix graph, BF16 weights and FP32
 * accumulation, trained on the GPU by its own forward, backward and Adam
 * kernels on (A, b, x_prev, x*) from solves of earlier steps.  The guess is
 * x_prev plus the network's correction; callers compare its residual with
 * the zero guess's and keep the better one.
 * ---------------------------------------------------------------------- */
typedef struct pg_mpnn pg_mpnn;
int pg_mpnn_create(uint64_t seed, pg_mpnn **out);
int pg_mpnn_destroy(pg_mpnn *net);
int pg_mpnn_num_params(const pg_mpnn *net);
/* graph = sparsity pattern of the systems (compact CSR, host arrays) */
int pg_mpnn_set_graph(pg_mpnn *net, const int32_t *row_ptr,
                      const int32_t *col_ind, int64_t n);
/* guess[n] from vals[nnz], b[n], x_prev[n]; *rel_residual (optional)
 * receives ||b - A guess|| / ||b|| (below 1: better than the zero guess). */
int pg_mpnn_predict(pg_mpnn *net, const double *vals, const double *b,
                    const double *x_prev, double *guess, double *rel_residual,
                    int ptr_kind);
/* one Adam step on one system; *loss (optional) = the normalised residual +
 * error loss of this step's forward pass */
int pg_mpnn_train_step(pg_mpnn *net, const double *vals, const double *b,
                       const double *x_prev, const double *x_star, float lr,
                       int ptr_kind, double *loss);
/* forward + backward only: the loss gradient with respect to the
 * parameters (pg_mpnn_num_params floats, host) and the loss */
int pg_mpnn_gradient(pg_mpnn *net, const double *vals, const double *b,
                     const double *x_prev, const double *x_star, int ptr_kind,
                     float *grad, double *loss);
/* FP32 master parameters (pg_mpnn_num_params floats), host memory */
int pg_mpnn_get_params(const pg_mpnn *net, float *params);
int pg_mpnn_set_params(pg_mpnn *net, const float *params);
/* Weights file: 8-byte tag "PGMPNN01", int32 parameter count, the FP32
 * master parameters (little-endian).  load checks the tag and the count
 * against this network's layout and resets the Adam state. */
int pg_mpnn_save(const pg_mpnn *net, const char *path);
int pg_mpnn_load(pg_mpnn *net, const char *path);

/* Allocation-free form of pg_gradient's cell gradient, for callers that
 * cannot allocate device memory (a fixed memory budget owned by an outer
 * framework, or code that must not let cudaMalloc/cudaFree synchronise the
 * device).  No counterpart in the reference.  All pointers are device
 * pointers: phi_cell[n_cells], phi_face[n_faces] in, grad_cell[2*n_cells]
 * out.  The face-gradient scratch is a static 16 MiB device array, so meshes
 * are limited to 1,048,576 faces (PG_BAD_ARG beyond).  One device: the
 * current device must be the mesh's, and the three pointers device memory
 * on it (PG_BAD_ARG otherwise).  The first call looks the array up (make it
 * before any stream capture); calls share the array, and calls that overlap
 * on the GPU race on it. */
int pg_gradient_noalloc(const pg_mesh *m, const double *phi_cell,
                        const double *phi_face, double *grad_cell);

/* ------------------------------------------------------------------------
 * Sparse solver.  Replaces the SparseMatrixSolver plugin
 * (src/Math/SparseMatrixSolver.h:11-62) as driven by
 * FiniteVolumeEquation<T>::solve (FiniteVolumeEquation.tpp:64-86), with
 * the semantics of the Belos BiCGStab + Ifpack2 right preconditioner backend
 * (TrilinosBelosSparseMatrixSolver.cpp:18-99, TrilinosSparseMatrixSolver.cpp
 * :23-112).
 * ---------------------------------------------------------------------- */
typedef struct {
  double tolerance;   /* ||b - A x||_2 / ||b||_2 target (Belos default 1e-8) */
  int max_iters;      /* Belos default 500 */
  int precond;        /* PG_PREC_* */
  int subdomain_rows; /* target rows per Schwarz subdomain; 0 = default
                         (1024; with the coarse correction 512, or
                         n / 2048 when larger); -1 = one subdomain
                         (global ILU(0)) */
  int precision;      /* PG_FP64 | PG_MIXED */
  int mixed_sweep;    /* PG_MIXED ILU(0) sweep form: 0 = timed choice at the
                         first factorisation, 1 = warp-wide steps, 2 = level
                         blobs, 3 = FP32-stored factor weights swept in
                         float-float arithmetic (the line form of
                         structured blocks; elsewhere as 0): half the factor
                         bytes, the factors rounded to FP32 */
  int coarse;         /* PG_PREC_ILU0: 0 = one-level Schwarz (as Ifpack2);
                         two-level, with a coarse space of subdomain-constant
                         vectors Z and y = (Z^T A Z)^-1 Z^T r (at most 2048
                         subdomains; pg_batch_*: a block per system, at most
                         4096 subdomains each):
                         1 = additive, M^-1 r = B r + Z y;
                         2 = deflated (A-DEF1), M^-1 r = B (r - A Z y) + Z y
                         (fewer iterations) */
  int coarse_warm;    /* one-level iterations a solve runs while the coarse
                         inverse is built beside them, before it restarts
                         with the two-level preconditioner: -1 = default (0
                         when the coarse inverse is built through the
                         sparse LU of the coarse matrix -- every front of
                         its nested dissection small, the usual case -- else
                         16 with at least 1024 subdomains), 0 = wait
                         for the inverse (when the caller already had work
                         to overlap it with after the hand-over), -2 = apply
                         the previous factorisation's inverse (same
                         pattern) for the whole solve while the new one is
                         built beside it, for the next solve (time loops,
                         where the coarse matrix changes little from step
                         to step; the first solve behaves as -1) */
  int krylov;         /* PG_KRYLOV_*: the Krylov method (BiCGStab default) */
  int ilu_fill;       /* level of fill k of the ILU blocks, Ifpack2 RILUK
                         "fact: iluk level-of-fill" (key iluFill,
                         TrilinosBelosSparseMatrixSolver.cpp:70): 0 = ILU(0) */
  int krylov_dim;     /* PG_KRYLOV_GMRES: Krylov vectors per restart cycle
                         (Belos "Num Blocks"); 0 = 300, Belos' default */
  int reserved_i;     /* ignored */
  double reserved_d;  /* ignored */
} pg_solver_cfg;

typedef struct {
  int iters;           /* BiCGStab iterations */
  int outer_iters;     /* reliable updates: true-residual replacements and
                          restarts */
  int status;          /* PG_OK, PG_MAX_ITERS, PG_BREAKDOWN, PG_NON_FINITE */
  int fp64_iters;      /* PG_MIXED: iterations of the FP64 solver that took
                          over from a stalled float-float solve (included in
                          iters); 0 otherwise */
  double rel_residual; /* true ||b - A x||_2 / ||b||_2 computed in FP64 */
  double ms;           /* device time of the solve (CUDA events) */
  double setup_ms;     /* device time the solve spent on (or waiting for)
                          the preconditioner factorisation; set_csr /
                          set_eqn start it on a side stream, so work issued
                          between the hand-over and the solve overlaps it */
} pg_solve_stats;

/* Defaults: tolerance 1e-8, max_iters 500, ILU(0) Schwarz, FP64. */
void pg_solver_default_cfg(pg_solver_cfg *cfg);
int pg_solver_create(const pg_solver_cfg *cfg, pg_solver **out);
int pg_solver_destroy(pg_solver *s);

/* SparseMatrixSolver::setRank(int) (SparseMatrixSolver.h:23). */
int pg_solver_set_rank(pg_solver *s, int64_t n);

/* SparseMatrixSolver::set(rowPtr, colInds, vals) (SparseMatrixSolver.h
 * :32-34).  Negative column indices are CrsEquation placeholders and are
 * skipped; repeated columns in a row are summed.  row_ptr[n+1],
 * col_ind[row_ptr[n]], vals[row_ptr[n]] in ptr_kind memory.  The sparsity
 * analysis (Schwarz partition, level schedule) is redone only when the
 * pattern differs from the previous call's. */
int pg_solver_set_csr(pg_solver *s, const int32_t *row_ptr,
                      const int32_t *col_ind, const double *vals,
                      int ptr_kind);

/* Optional geometry hint for pg_solver_set_csr: a point per row (for a
 * finite-volume system the cell centroids, FiniteVolumeGrid2D's
 * cells()[i].centroid()), host xy[2n] interleaved.  Later analyses cut the
 * Schwarz subdomains by coordinate bisection, as pg_solver_set_eqn does
 * with its mesh, instead of by graph distance.  NULL clears the hint.
 * Call after pg_solver_set_rank.  (No reference counterpart: the
 * SparseMatrixSolver interface carries no geometry.) */
int pg_solver_set_row_coords(pg_solver *s, const double *xy);

/* Take the matrix and -rhs_ of a device equation without a host round trip
 * (the device form of FiniteVolumeEquation::solve's set + setRhs). */
int pg_solver_set_eqn(pg_solver *s, const pg_eqn *e);

/* The same for one component of a momentum equation (component 0: the x
 * rows, 1: the y rows; VectorFiniteVolumeEquation::solve solves the rank-2N
 * system whose two diagonal blocks are this one matrix,
 * src/2D/Unstructured/FiniteVolume/Equation/VectorFiniteVolumeEquation.cpp
 * :5-30,129-146); component 0 for any other equation.  Handing over a
 * component of the same equation at the same assembly as the previous
 * call replaces only the right-hand side and keeps the factorisation
 * (pg_solver_set_eqn always factors anew). */
int pg_solver_set_eqn_component(pg_solver *s, const pg_eqn *e, int component);

/* SparseMatrixSolver::setRhs (receives the already negated rhs) and
 * setGuess (SparseMatrixSolver.h:38-40).  rhs[n], x0[n]; x0 == NULL sets a
 * zero initial guess. */
int pg_solver_set_rhs(pg_solver *s, const double *rhs, int ptr_kind);
int pg_solver_set_guess(pg_solver *s, const double *x0, int ptr_kind);

/* SparseMatrixSolver::solve (SparseMatrixSolver.h:42): factor the
 * preconditioner and iterate from the current guess (the previous solution
 * unless set_guess was called, as Belos' warm start).  Blocks until done. */
int pg_solver_solve(pg_solver *s, pg_solve_stats *stats);

/* SparseMatrixSolver::x(i) for all i (SparseMatrixSolver.h:48). x[n]. */
int pg_solver_get_x(const pg_solver *s, double *x, int ptr_kind);

/* Time the solver's kernels in isolation on its current system: each is
 * launched `reps` times back to back on the library stream between CUDA
 * events, on scratch vectors.  Per launch, ms[0] FP64 SpMV with fused dot,
 * ms[1] FP64 ILU(0)/Jacobi apply with fused update, ms[2] FP64 BiCGStab x/r
 * update, ms[3] ILU(0) factorisation (with the coarse matrix and its
 * inverse when cfg.coarse), for PG_MIXED ms[4] the float-float ILU(0)
 * apply, ms[5] SpMV and ms[6] update (0 otherwise), and ms[7] the coarse
 * stage of one application (0 without a coarse space): for cfg.coarse = 1
 * the subdomain sums and the correction z += Z y, for cfg.coarse = 2 the
 * deflation's kernels beside the sweep (the combined input with its
 * subdomain sums, y = A_c^-1 Z^T p and p - A Z y; float-float ones under
 * PG_MIXED), ms[8] the coarse matrix's assembly and inversion alone (0
 * without a coarse space).  Leaves the solver's state untouched.  (No
 * reference counterpart: measurement.) */
int pg_solver_profile(pg_solver *s, int reps, double *ms);

/* Kernel time inside a solve (no reference counterpart: measurement).
 * With on != 0 the BiCGStab solves that follow launch their iteration
 * chunks directly instead of replaying CUDA graphs, with a CUDA event on
 * the library stream after every launch group; pg_solver_kernel_times then
 * returns, for the last such solve, the device time ms[k] (milliseconds)
 * and the number count[k] of groups of each kind k below, and in *dropped
 * (may be NULL) the groups left untimed when the event pool (65,536) ran
 * out.  Intervals that span a host wait (chunk boundaries) are not booked.
 * Synchronises the library stream. */
#define PG_KT_SPMV 0   /* SpMV with its fused dot products */
#define PG_KT_SWEEP 1  /* preconditioner sweep (ILU(k) or Jacobi) */
#define PG_KT_UPDATE 2 /* x / r update with its fused dot products */
#define PG_KT_COARSE 3 /* coarse correction: the deflation stage before the
                          sweep (input sums, y = A_c^-1 Z^T p, p - A Z y), or
                          the additive correction after it */
#define PG_KT_N 4
int pg_solver_trace_kernels(pg_solver *s, int on);
int pg_solver_kernel_times(pg_solver *s, double *ms, int64_t *count,
                           int64_t *dropped);

/* ---------------------------------------------------------------------
 * Batched solves: many independent pressure systems of uneven sizes
 * (e.g. one per immersed-boundary case) solved together.  The reference
 * solves them one FiniteVolumeEquation::solve() at a time
 * (FiniteVolumeEquation.tpp:64-86); here they share one analysis, one
 * ILU(0) factorisation launch and one CUDA graph launch for the whole
 * BiCGStab iteration, with per-system scalars, convergence and statistics.
 * FP64, Schwarz ILU(0) (the cfg's subdomain size applies per system), zero
 * initial guess.  The tile shape of the row kernels is autotuned per batch
 * pattern.
 * --------------------------------------------------------------------- */
typedef struct pg_batch pg_batch;
int pg_batch_create(const pg_solver_cfg *cfg, pg_batch **out);
int pg_batch_destroy(pg_batch *b);
/* Device equations, one per system (values and -rhs_ are copied at this
 * call; a new list of patterns triggers a new analysis and autotuning). */
int pg_batch_set_eqns(pg_batch *b, int n_systems, const pg_eqn *const *eqns);
/* stats[n_systems] (may be NULL); ms_total: device time of the batch solve
 * (factorisation included).  Returns PG_OK when every system converged on
 * its FP64 true residual, else the first failing status. */
int pg_batch_solve(pg_batch *b, pg_solve_stats *stats, double *ms_total);
/* solution of one system, in its own row order */
int pg_batch_get_x(const pg_batch *b, int system, double *x, int ptr_kind);
/* the autotuned tile shape: threads per CTA, rows per thread, tile count */
int pg_batch_tuning(const pg_batch *b, int *block, int *rows_per_thread,
                    int *n_tiles);

/* ---------------------------------------------------------------------
 * Direct sparse solve.  Replaces the SparseMatrixSolver backend that most
 * of Phase's cases select for the pressure equation (`lib eigen`):
 * EigenSparseMatrixSolver (src/Math/EigenSparseMatrixSolver.cpp:5-64),
 * whose set() builds the matrix from the entries with col >= 0 (repeated
 * entries summed, :17-48) and whose solve() factorises and solves on every
 * call (SparseLU::compute + solve, :60-64), reporting nIters() = 1 and
 * error() = 0 (EigenSparseMatrixSolver.h:43-45).  Here: a multifrontal LU
 * over a nested-dissection ordering (cut by the row coordinates when given,
 * by graph bisection otherwise), FP64, partial pivoting inside the fully
 * summed rows of each front (32-row blocks of the larger fronts); the
 * ordering and front structure are computed once per pattern, the numeric
 * factorisation on every solve after new values (as the reference's
 * compute), and a solve with only a new right-hand side reuses the
 * factors.  A pivot at most 1e-13 of its column's largest entry in A is
 * replaced by that entry and counted (replaced_pivots): a consistent
 * singular system (all-Neumann pressure) gets one of its solutions.
 * --------------------------------------------------------------------- */
typedef struct pg_lu pg_lu;
typedef struct {
  int n_fronts;           /* nodes of the nested-dissection tree */
  int n_heights;          /* levels of fronts factorised one after another */
  int max_front;          /* order of the largest front */
  int replaced_pivots;    /* vanishing pivots replaced (see above) */
  int64_t factor_entries; /* entries of L and U */
  double flops;           /* factorisation flops (multiply-add = 2) */
  double analyse_ms;      /* host time of the last ordering + symbolic */
  double factor_ms;       /* device time of the last factorisation */
  double solve_ms;        /* device time of the last triangular solves */
  double rel_residual;    /* ||b - A x||_2 / ||b||_2 computed in FP64 */
} pg_lu_stats;
int pg_lu_create(pg_lu **out);
int pg_lu_destroy(pg_lu *lu);
/* setRank (EigenSparseMatrixSolver.cpp:5-9) */
int pg_lu_set_rank(pg_lu *lu, int64_t n);
/* optional point per row (xy[2 n], e.g. cell centres) for the ordering;
 * NULL clears it */
int pg_lu_set_row_coords(pg_lu *lu, const double *xy);
/* set(rowPtr, colInds, vals) (EigenSparseMatrixSolver.cpp:31-40): entries
 * with a negative column are skipped, repeated columns summed */
int pg_lu_set_csr(pg_lu *lu, const int32_t *row_ptr, const int32_t *col_ind,
                  const double *vals, int ptr_kind);
/* the matrix and -rhs_ of a device equation (FiniteVolumeEquation::solve's
 * setRank + set + setRhs, FiniteVolumeEquation.tpp:71-73), cells' centres
 * as the ordering's coordinates */
int pg_lu_set_eqn(pg_lu *lu, const pg_eqn *e);
/* setRhs (EigenSparseMatrixSolver.cpp:55-58) */
int pg_lu_set_rhs(pg_lu *lu, const double *rhs, int ptr_kind);
/* solve (EigenSparseMatrixSolver.cpp:60-64); stats may be NULL */
int pg_lu_solve(pg_lu *lu, pg_lu_stats *stats);
/* x (EigenSparseMatrixSolver.h:39) for all rows */
int pg_lu_get_x(const pg_lu *lu, double *x, int ptr_kind);
/* The ordering and front structure alone (host work, no GPU needed), for
 * inspection: sizes[4] = {fronts, index-list length, heights, largest
 * front}; when the arrays are non-NULL also perm[n] (elimination order:
 * new -> old row), fronts[4 * n_fronts] = (first new index, fully summed
 * count k, order m, parent or -1) in elimination order, and fidx[] (each
 * front's index list: its k own rows, then its update rows ascending).
 * xy: optional point per row; leaf: largest vertex set that is not cut
 * (0: the solver's default, 64).  (Inspection; no reference counterpart.) */
int pg_lu_analyse_pattern(int64_t n, const int32_t *row_ptr,
                          const int32_t *col_ind, const double *xy, int leaf,
                          int64_t *sizes, int32_t *perm, int32_t *fronts,
                          int32_t *fidx);

/* Number of kernels the library has launched since it was loaded. */
uint64_t pg_kernel_launches(void);

/* The form of the ILU(0) sweep the solver runs on its current analysis: 1
 * the line form (every Schwarz subdomain a rectangular block of a structured
 * grid: one grid line per lane, levels carried by warp shuffles, no column
 * indices read), 0 the stream form (level blobs with 2-byte columns), -1 no
 * ILU(0) sweep (another preconditioner, or nothing analysed).
 * (Inspection; no reference counterpart.) */
int pg_solver_sweep_form(const pg_solver *s);

/* Subdomain id of every row of the last analysed pattern (host, part[n]);
 * returns the number of subdomains in *n_parts. */
int pg_solver_partition(const pg_solver *s, int32_t *part, int *n_parts);

/* The two-level preconditioner's coarse inverse (cfg.coarse = 1 or 2) of
 * the last factorisation (an inversion still running is joined first): the
 * K x K row-major FP32 approximation of
 * (Z^T A Z)^-1 that the solver applies, K = *n_parts of pg_solver_partition
 * and Z the subdomain indicator vectors (host, out[K*K]).  Returns
 * PG_INVALID_ARG when no coarse space is active.  (Inspection; no reference
 * counterpart.) */
int pg_solver_coarse_inverse(pg_solver *s, float *out, int *k);

/* z = M^-1 r for the solver's preconditioner on its current matrix (the
 * ILU(0) factors are recomputed from the current values; FP32 factors and
 * sweeps under PG_MIXED), r and z in the caller's row order.  The Ifpack2
 * preconditioner's apply() (TrilinosBelosSparseMatrixSolver.cpp:63-85, used
 * by Belos inside the iteration); exposed for parity checks of the sweeps.
 * Overwrites the solver's Krylov work vectors but not its solution. */
int pg_solver_apply_precond(pg_solver *s, const double *r, double *z,
                            int ptr_kind);

#ifdef __cplusplus
}
#endif

#endif
