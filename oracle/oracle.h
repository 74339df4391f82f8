/*
 * CPU oracle for the Phase pressure-solve path -- TEST INFRASTRUCTURE ONLY.
 *
 * This library restates, in plain C++, the reference algorithms that the
 * GB300 library replaces.  It is used by the tests, by the CPU baseline leg
 * of bench.py and by __graft_entry__.smoke() as the checker.  Nothing in the
 * product (phase_gb300/) links against it or calls it.
 *
 * Each function cites the reference file:line it follows (paths relative to
 * the obrienadam/Phase source tree).
 *
 * Parity status: the CSR container semantics are pinned against the
 * reference's own src/Math/CrsEquation.cpp compiled into oracle/_ref (see
 * oracle/Makefile); mesh geometry, assembly and the Krylov solve are pinned
 * against known-answer tests (rectilinear coefficients, zero Laplacian of
 * linear fields, row sums) and scipy cross-checks, because the reference's
 * own tests pin nothing on this path and its solver libraries (Eigen,
 * Trilinos) are not available.
 */
#ifndef PHASE_ORACLE_H
#define PHASE_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Boundary condition codes, as FiniteVolumeField<T>::BoundaryType
 * (src/2D/Unstructured/FiniteVolume/Field/FiniteVolumeField.h). */
enum { OR_FIXED = 0, OR_NORMAL_GRADIENT = 1, OR_SYMMETRY = 2 };

typedef struct or_mesh or_mesh;
typedef struct or_eqn or_eqn;

/* ---- mesh (FiniteVolumeGrid2D::init, createCell, init links) ---- */
or_mesh *or_mesh_create(const double *nodes_xy, int64_t n_nodes,
                        const int64_t *cptr, const int64_t *cind,
                        int64_t n_cells);
void or_mesh_destroy(or_mesh *m);
void or_mesh_sizes(const or_mesh *m, int64_t *n_cells, int64_t *n_faces,
                   int64_t *n_interior, int64_t *n_boundary);
/* per cell: centroid x,y and volume */
void or_mesh_cells(const or_mesh *m, double *cx, double *cy, double *vol);
/* per face: lCell, rCell (-1 if boundary), lNode, rNode, centroid, normal
 * (= normalVec() of rNode - lNode) */
void or_mesh_faces(const or_mesh *m, int32_t *lcell, int32_t *rcell,
                   int32_t *lnode, int32_t *rnode, double *fx, double *fy,
                   double *nx, double *ny);
/* per cell links in reference order: interior links then boundary links.
 * link_ptr[n_cells+1], link_face[], link_cell[] (-1 for boundary links) */
int64_t or_mesh_nlinks(const or_mesh *m);
void or_mesh_links(const or_mesh *m, int64_t *link_ptr, int32_t *link_face,
                   int32_t *link_cell);

/* ---- fields ---- */
/* FiniteVolumeField::interpolateFaces(DISTANCE) + setBoundaryFaces for a
 * NORMAL_GRADIENT-everywhere field: out[face] */
void or_interpolate_faces(const or_mesh *m, const double *cell_vals,
                          double *face_vals);
/* dt / rho_f with rho_f = rho1 + clamp(gamma_f,0,1)*(rho2-rho1)
 * (FractionalStepMultiphase.cpp:175-185, ScalarFiniteVolumeField.cpp:68-81) */
void or_dt_over_rho_faces(const or_mesh *m, const double *gamma_face,
                          double rho1, double rho2, double dt, double *out);

/* ---- assembly ---- */
/* fv::laplacian(gamma, phi) (Laplacian.h:49-83 scalar gamma, :132-167 face
 * field gamma) == src::div(u) (Source.cpp:5-25) with CrsEquation semantics
 * (CrsEquation.cpp:9-14 ctor, :113-131 addCoeff, :282-285,309-311
 * operator==(Vector)).
 * gamma_face NULL -> scalar gamma overload.  u_face_xy NULL -> no div term.
 * bc_type/bc_value indexed by face id (only boundary faces are read). */
or_eqn *or_laplacian(const or_mesh *m, const double *gamma_face,
                     double gamma_scalar, const int32_t *bc_type,
                     const double *bc_value, const double *u_face_xy);
void or_eqn_destroy(or_eqn *e);
/* n rows, number of slots (incl. -1 placeholders), number of used entries */
void or_eqn_sizes(const or_eqn *e, int64_t *n, int64_t *n_slots,
                  int64_t *nnz);
/* raw CrsEquation arrays exactly as FiniteVolumeEquation::solve hands them
 * to SparseMatrixSolver::set (with -1 placeholders), and rhs_ */
void or_eqn_export_slots(const or_eqn *e, int32_t *row_ptr, int32_t *col_ind,
                         double *vals, double *rhs);
/* compact CSR (placeholders dropped, order kept) */
void or_eqn_export_csr(const or_eqn *e, int32_t *row_ptr, int32_t *col_ind,
                       double *vals, double *rhs);

/* ScalarGradient::computeFaces + compute(FACE_TO_CELL)
 * (ScalarGradient.cpp:34-74).  phi_face holds boundary face values. */
void or_gradient(const or_mesh *m, const double *phi_cell,
                 const double *phi_face, double *grad_face_xy,
                 double *grad_cell_xy);

/* ---- Krylov solve ---- */
enum { OR_PREC_NONE = 0, OR_PREC_JACOBI = 1, OR_PREC_ILU0 = 2,
       OR_PREC_ILUT = 3 };

typedef struct {
  double tol;          /* ||b - A x||_2 / ||b||_2 stop threshold */
  int max_iters;
  int precond;         /* OR_PREC_* */
  double ilut_drop;    /* ILUT drop tolerance (relative to row 2-norm) */
  int ilut_fill;       /* ILUT extra entries kept per row in L and in U */
  int n_threads;       /* OpenMP threads (0 = default) */
  const int32_t *part; /* optional subdomain id per row (additive Schwarz,
                          overlap 0); NULL = one global subdomain */
  int n_parts;
  int use_guess;       /* 1: x holds the initial guess; 0: zero guess */
  int coarse;          /* with part: 0 one-level Schwarz; two-level with the
                          subdomain-constant coarse space Z (A_c = Z^T A Z,
                          dense LU with partial pivoting): 1 additive
                          M^-1 r = B r + Z A_c^-1 Z^T r, 2 deflated (A-DEF1)
                          M^-1 r = B (r - A Z y) + Z y, y = A_c^-1 Z^T r */
  int krylov;          /* 0 BiCGStab, 1 TFQMR, 2 GMRES (Belos "solver",
                          TrilinosBelosSparseMatrixSolver.cpp:59-60) */
  int krylov_dim;      /* GMRES restart length (0 = 300, Belos' default) */
  int ilu_fill;        /* OR_PREC_ILU0 blocks: level of fill k (ILU(k),
                          Ifpack2 RILUK "fact: iluk level-of-fill") */
} or_solver_cfg;

typedef struct {
  int iters;
  int status; /* 0 converged, 1 max iters, 2 breakdown, 3 non-finite */
  double rel_residual; /* true ||b-Ax||/||b|| at exit */
  double ms;
  double setup_ms;
} or_solver_stats;

/* BiCGStab right-preconditioned, as Belos BICGSTAB with an Ifpack2
 * schwarz/RILUK right preconditioner (TrilinosBelosSparseMatrixSolver.cpp
 * :18-29,44-86).  CSR must be compact (no negative columns). */
int or_bicgstab(int64_t n, const int32_t *row_ptr, const int32_t *col_ind,
                const double *vals, const double *b, double *x,
                const or_solver_cfg *cfg, or_solver_stats *stats);

/* Run at most max_iters iterations and record the recursive residual norm
 * ||r_k|| / ||b|| after every iteration into hist[0..max_iters]; returns the
 * number of iterations run.  Used by the CPU baseline to time a bounded
 * sample of a long solve. */
int or_bicgstab_history(int64_t n, const int32_t *row_ptr,
                        const int32_t *col_ind, const double *vals,
                        const double *b, const or_solver_cfg *cfg,
                        double *hist, double *ms_out, double *setup_ms_out);
/* The same from the initial guess x0[n] (NULL: zero), as a time loop's
 * solve warm from the previous step's solution. */
int or_bicgstab_history_x0(int64_t n, const int32_t *row_ptr,
                           const int32_t *col_ind, const double *vals,
                           const double *b, const double *x0,
                           const or_solver_cfg *cfg, double *hist,
                           double *ms_out, double *setup_ms_out);

/* z = (LU)^-1 r with the ILU(k) factor (level of fill k) of each subdomain
 * (part, or one subdomain when NULL) of a compact CSR; returns 0, or 2 on a
 * zero pivot. */
int or_iluk_apply(int64_t n, const int32_t *row_ptr, const int32_t *col_ind,
                  const double *vals, const int32_t *part, int fill,
                  const double *r, double *z);

/* ILU(0) factor in place on a compact CSR (per subdomain when part given);
 * out_vals receives the L (unit, strictly lower) and U values in the CSR
 * pattern of A restricted to each subdomain (entries that leave the
 * subdomain are written as 0). */
int or_ilu0(int64_t n, const int32_t *row_ptr, const int32_t *col_ind,
            const double *vals, const int32_t *part, double *out_vals);
/* z = M^-1 r for the ILU(0) factors above */
void or_ilu0_apply(int64_t n, const int32_t *row_ptr, const int32_t *col_ind,
                   const double *lu_vals, const int32_t *part,
                   const double *r, double *z);

/* Momentum operator of the vector equation
 *   fv::ddt(u, dt) + fv::div(uf, u, theta) - fv::laplacian(nu, u, theta)
 * (TimeDerivative.h:38-48, Divergence.h:8-53, Laplacian.h:7-47) combined
 * with CrsEquation::operator+= / -= (CrsEquation.cpp:185-275, which drop
 * zero and placeholder entries).  Rows 0..N-1 are the x component, N..2N-1
 * the y component (VectorFiniteVolumeEquation.cpp:5-30); both share the
 * coefficients.  u_old_cell[2N] (x,y per cell), u_face[2F] face velocity
 * for the fluxes and for FIXED boundary values, bc_type per face.  Returns
 * the equation (2N rows) for or_eqn_sizes / or_eqn_export_csr. */
or_eqn *or_momentum(const or_mesh *m, double dt, double nu, double theta,
                    const double *u_old_cell, const double *u_face,
                    const int32_t *bc_type);
/* Ghost-cell immersed-boundary pressure equation
 *   (fv::laplacian(gamma, p) + ib.bcs(p)) == src::div(u)
 * (FractionalStepGCIB.cpp:44-46, GhostCellImmersedBoundary.cpp:12-74,
 * GhostCellImmersedBoundary*BcStencil.cpp) for circles[3k..3k+2] =
 * (cx, cy, r); ib_bc OR_FIXED or OR_NORMAL_GRADIENT with reference value
 * ib_ref.  cell_class[n] (optional) receives 0 fluid, 1 IB, 2 solid.
 * Returns NULL when a stencil is degenerate. */
or_eqn *or_gcib_laplacian(const or_mesh *m, const double *gamma_face,
                          double gamma_scalar, const int32_t *bc_type,
                          const double *bc_value, const double *u_face_xy,
                          int n_circles, const double *circles, int ib_bc,
                          double ib_ref, int32_t *cell_class);
/* FiniteVolumeField::setBoundaryFaces: faces of NORMAL_GRADIENT/SYMMETRY
 * boundaries take their cell's value (FiniteVolumeField.tpp:165-183). */
void or_set_boundary_faces(const or_mesh *m, const int32_t *bc_type,
                           const double *phi_cell, double *phi_face);
/* FractionalStep::correctVelocity: u -= dt / rho * grad p on cells and
 * faces (FractionalStep.cpp:109-117, FractionalStepMultiphase.cpp:165-173);
 * rho arrays NULL = 1.  x,y interleaved. */
void or_correct_velocity(const or_mesh *m, double dt, const double *rho_cell,
                         const double *rho_face, const double *grad_cell,
                         const double *grad_face, double *u_cell,
                         double *u_face);
/* y = A x */
void or_spmv(int64_t n, const int32_t *row_ptr, const int32_t *col_ind,
             const double *vals, const double *x, double *y);

/* Direct solve of the matrix of the entries with col >= 0 (repeated
 * entries summed): band LU with partial pivoting in a reverse Cuthill-McKee
 * order (EigenSparseMatrixSolver.cpp:17-64 semantics).  band[2] receives the
 * (lower, upper) bandwidths, *replaced the vanishing pivots replaced. */
int or_sparse_lu_solve(int64_t n, const int32_t *row_ptr, const int32_t *col_ind,
                       const double *vals, const double *b, double *x,
                       int64_t *band, int *replaced);

#ifdef __cplusplus
}
#endif

#endif
