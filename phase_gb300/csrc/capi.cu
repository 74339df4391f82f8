// C ABI of libphase_gb300 (include/phase_gb300.h) and the host drivers of
// the mesh, the device equation and the BiCGStab solver.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "internal.h"
#include "kernels.cuh"

namespace pg {

static thread_local std::string g_err;

void set_error(const std::string &msg) { g_err = msg; }

int cuda_fail(cudaError_t e, const char *what, const char *file, int line) {
  g_err = std::string("CUDA error ") + cudaGetErrorName(e) + " (" +
          cudaGetErrorString(e) + ") in " + what + " at " + file + ":" +
          std::to_string(line);
  return PG_CUDA_ERROR;
}

cudaStream_t stream() {
  static cudaStream_t s = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess)
      s = nullptr;
  });
  return s;
}

cudaError_t copy_in(void *dst, const void *src, size_t bytes, int ptr_kind) {
  if (!bytes) return cudaSuccess;
  return cudaMemcpyAsync(dst, src, bytes,
                         ptr_kind == PG_DEVICE ? cudaMemcpyDeviceToDevice
                                               : cudaMemcpyHostToDevice,
                         stream());
}

cudaError_t copy_out(void *dst, const void *src, size_t bytes, int ptr_kind) {
  if (!bytes) return cudaSuccess;
  return cudaMemcpyAsync(dst, src, bytes,
                         ptr_kind == PG_DEVICE ? cudaMemcpyDeviceToDevice
                                               : cudaMemcpyDeviceToHost,
                         stream());
}

// Make `src` usable as a device pointer: device pointers pass through, host
// arrays are staged into `buf`.
template <class T>
static int stage(const T *src, size_t count, int ptr_kind, DevBuf<T> &buf,
                 const T **out) {
  if (!src) {
    *out = nullptr;
    return PG_OK;
  }
  if (ptr_kind == PG_DEVICE) {
    *out = src;
    return PG_OK;
  }
  PG_CUDA(buf.upload(src, count));
  *out = buf.p;
  return PG_OK;
}

static int check_device() {
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) {
    set_error("no CUDA device available: libphase_gb300 has no CPU path");
    return PG_CUDA_ERROR;
  }
  if (!stream()) {
    set_error("could not create the library CUDA stream");
    return PG_CUDA_ERROR;
  }
  return PG_OK;
}

}  // namespace pg

using namespace pg;

// ------------------------------------------------------------------ misc
extern "C" const char *pg_last_error(void) { return g_err.c_str(); }

extern "C" void *pg_stream(void) { return (void *)stream(); }

extern "C" int pg_synchronize(void) {
  PG_CUDA(cudaStreamSynchronize(stream()));
  return PG_OK;
}

// ------------------------------------------------------------------ mesh
extern "C" int pg_mesh_create(const double *nodes_xy, int64_t n_nodes,
                              const int64_t *cptr, const int64_t *cind,
                              int64_t n_cells, pg_mesh **out) {
  PG_CHECK_ARG(out, "pg_mesh_create: out is NULL");
  *out = nullptr;
  int rc = check_device();
  if (rc) return rc;
  auto *m = new (std::nothrow) pg_mesh();
  PG_CHECK_ARG(m, "pg_mesh_create: out of host memory");
  rc = build_host_mesh(nodes_xy, n_nodes, cptr, cind, n_cells, m->h);
  if (rc) {
    delete m;
    return rc;
  }
  const HostMesh &h = m->h;
  const int64_t nf = h.n_faces;
  // per face side geometry of the links (InteriorLink.cpp:6-10,
  // BoundaryLink.cpp:6-10, Face::outwardNorm Face.cpp:48-50)
  m->dot_l.resize(nf);
  m->dot_r.assign(nf, 0.);
  m->msq.resize(nf);
  m->sgn_l.resize(nf);
  m->sgn_r.assign(nf, 0);
  auto outward = [&](int64_t f, double px, double py) -> int8_t {
    const double d = (h.fcx[f] - px) * h.fnx[f] + (h.fcy[f] - py) * h.fny[f];
    return d > 0. ? 1 : -1;
  };
  for (int64_t f = 0; f < nf; ++f) {
    const int32_t l = h.fl[f], r = h.fr[f];
    const int8_t sl = outward(f, h.cx[l], h.cy[l]);
    const double slx = sl * h.fnx[f], sly = sl * h.fny[f];
    m->sgn_l[f] = sl;
    if (r >= 0) {
      const double rx = h.cx[r] - h.cx[l], ry = h.cy[r] - h.cy[l];
      m->dot_l[f] = rx * slx + ry * sly;
      m->msq[f] = rx * rx + ry * ry;
      const int8_t sr = outward(f, h.cx[r], h.cy[r]);
      m->sgn_r[f] = sr;
      const double qx = h.cx[l] - h.cx[r], qy = h.cy[l] - h.cy[r];
      m->dot_r[f] = qx * (sr * h.fnx[f]) + qy * (sr * h.fny[f]);
    } else {
      const double rx = h.fcx[f] - h.cx[l], ry = h.fcy[f] - h.cy[l];
      m->dot_l[f] = rx * slx + ry * sly;
      m->msq[f] = rx * rx + ry * ry;
    }
  }
  DevMesh &d = m->d;
  cudaError_t e = cudaSuccess;
  auto up = [&](auto &buf, const auto &vec) {
    if (e == cudaSuccess) e = buf.upload(vec);
  };
  up(d.cx, h.cx);
  up(d.cy, h.cy);
  up(d.vol, h.vol);
  up(d.fl, h.fl);
  up(d.fr, h.fr);
  up(d.fcx, h.fcx);
  up(d.fcy, h.fcy);
  up(d.fnx, h.fnx);
  up(d.fny, h.fny);
  up(d.link_ptr, h.link_ptr);
  up(d.link_face, h.link_face);
  if (e == cudaSuccess) e = d.fw.reserve(nf);
  if (e == cudaSuccess) {
    launch_face_weights((int)nf, d.fl.p, d.fr.p, d.fcx.p, d.fcy.p, d.cx.p,
                        d.cy.p, d.fw.p, stream());
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(stream());
  if (e != cudaSuccess) {
    delete m;
    return cuda_fail(e, "mesh upload", __FILE__, __LINE__);
  }
  *out = m;
  return PG_OK;
}

extern "C" int pg_mesh_destroy(pg_mesh *m) {
  delete m;
  return PG_OK;
}

extern "C" int pg_mesh_sizes(const pg_mesh *m, int64_t *n_cells,
                             int64_t *n_faces, int64_t *n_interior,
                             int64_t *n_boundary) {
  PG_CHECK_ARG(m, "pg_mesh_sizes: NULL mesh");
  if (n_cells) *n_cells = m->h.n_cells;
  if (n_faces) *n_faces = m->h.n_faces;
  if (n_interior) *n_interior = m->h.n_interior;
  if (n_boundary) *n_boundary = m->h.n_boundary;
  return PG_OK;
}

extern "C" int pg_mesh_faces(const pg_mesh *m, int32_t *lcell, int32_t *rcell,
                             double *fx, double *fy, double *nx, double *ny) {
  PG_CHECK_ARG(m, "pg_mesh_faces: NULL mesh");
  const HostMesh &h = m->h;
  auto cp = [&](auto *dst, const auto &v) {
    if (dst) std::copy(v.begin(), v.end(), dst);
  };
  cp(lcell, h.fl);
  cp(rcell, h.fr);
  cp(fx, h.fcx);
  cp(fy, h.fcy);
  cp(nx, h.fnx);
  cp(ny, h.fny);
  return PG_OK;
}

extern "C" int pg_mesh_cells(const pg_mesh *m, double *cx, double *cy,
                             double *vol) {
  PG_CHECK_ARG(m, "pg_mesh_cells: NULL mesh");
  const HostMesh &h = m->h;
  if (cx) std::copy(h.cx.begin(), h.cx.end(), cx);
  if (cy) std::copy(h.cy.begin(), h.cy.end(), cy);
  if (vol) std::copy(h.vol.begin(), h.vol.end(), vol);
  return PG_OK;
}

// -------------------------------------------------------------- equation
static uint64_t next_pattern_id() {
  static std::mutex mu;
  static uint64_t id = 0;
  std::lock_guard<std::mutex> g(mu);
  return ++id;
}

static int eqn_create(const pg_mesh *m, int gamma_kind, const int32_t *bc_type,
                      bool momentum, pg_eqn **out, const GcibRows *ib = nullptr);

extern "C" int pg_eqn_create(const pg_mesh *m, int gamma_kind,
                             const int32_t *bc_type, pg_eqn **out) {
  return eqn_create(m, gamma_kind, bc_type, false, out);
}

extern "C" int pg_eqn_create_momentum(const pg_mesh *m, const int32_t *bc_type,
                                      pg_eqn **out) {
  return eqn_create(m, PG_GAMMA_FACE, bc_type, true, out);
}

// Fills e (new, or a ghost-cell IB equation whose pattern changed) with
// the pattern, the face schedule and the constant rows; bc_type must not
// alias e->bc_type.
static int eqn_fill(pg_eqn *e, const pg_mesh *m, int gamma_kind,
                    const int32_t *bc_type, bool momentum, const GcibRows *ib) {
  const HostMesh &h = m->h;
  e->mesh = m;
  e->gamma_kind = gamma_kind;
  e->bc_type.assign(bc_type, bc_type + h.n_faces);
  e->momentum = momentum;
  int rc = build_pattern(h, gamma_kind, bc_type, e->p, momentum, ib);
  if (rc) return rc;
  e->pattern_id = next_pattern_id();
  e->any_fixed = false;
  for (int64_t f = 0; f < h.n_faces && !e->any_fixed; ++f)
    e->any_fixed = h.fr[f] < 0 && bc_type[f] == PG_BC_FIXED;
  const EqnPattern &p = e->p;
  const int64_t nf = h.n_faces;
  std::vector<int32_t> cl(nf), cr(nf), cbc(nf);
  std::vector<double> dl(nf), dr(nf), ms(nf), slx(nf), sly(nf), srx(nf),
      sry(nf);
  for (int64_t k = 0; k < nf; ++k) {
    const int32_t f = p.cface[k];
    // a side whose cell is not fluid (ghost-cell IB) gets no Laplacian or
    // source contribution: the kernels skip sides with cell -1
    cl[k] = ib && ib->cls[h.fl[f]] != 0 ? -1 : h.fl[f];
    cr[k] = ib && h.fr[f] >= 0 && ib->cls[h.fr[f]] != 0 ? -1 : h.fr[f];
    cbc[k] = h.fr[f] < 0 ? bc_type[f] : -1;
    dl[k] = m->dot_l[f];
    dr[k] = m->dot_r[f];
    ms[k] = m->msq[f];
    slx[k] = m->sgn_l[f] * h.fnx[f];
    sly[k] = m->sgn_l[f] * h.fny[f];
    srx[k] = m->sgn_r[f] * h.fnx[f];
    sry[k] = m->sgn_r[f] * h.fny[f];
  }
  cudaError_t ce = cudaSuccess;
  auto up = [&](auto &buf, const auto &vec) {
    if (ce == cudaSuccess) ce = buf.upload(vec);
  };
  up(e->row_ptr, p.row_ptr);
  up(e->col_ind, p.col_ind);
  up(e->cface, p.cface);
  up(e->cl, cl);
  up(e->cr, cr);
  up(e->cbc, cbc);
  up(e->slot_lr, p.slot_lr);
  up(e->slot_rl, p.slot_rl);
  up(e->diag_l, p.diag_l);
  up(e->diag_r, p.diag_r);
  up(e->cdot_l, dl);
  up(e->cdot_r, dr);
  up(e->cmsq, ms);
  up(e->csfl_x, slx);
  up(e->csfl_y, sly);
  up(e->csfr_x, srx);
  up(e->csfr_y, sry);
  up(e->diag, p.diag);
  if (ib) {
    // constant IB and solid rows: the assembly starts from these values
    std::vector<double> bv(p.nnz, 0.);
    for (int64_t c = 0; c < p.n; ++c)
      for (const auto &en : ib->rows[c])
        for (int32_t q = p.row_ptr[c]; q < p.row_ptr[c + 1]; ++q)
          if (p.col_ind[q] == en.first) {
            bv[q] = en.second;
            break;
          }
    up(e->base_vals, bv);
    up(e->base_rhs, ib->rhs);
    e->cell_class = ib->cls;
    e->has_base = true;
  }
  if (ce == cudaSuccess) ce = e->vals.zero(p.nnz);
  if (ce == cudaSuccess) ce = e->rhs.zero(momentum ? 2 * p.n : p.n);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(stream());
  if (ce != cudaSuccess) return cuda_fail(ce, "equation upload", __FILE__, __LINE__);
  return PG_OK;
}

static int eqn_create(const pg_mesh *m, int gamma_kind, const int32_t *bc_type,
                      bool momentum, pg_eqn **out, const GcibRows *ib) {
  PG_CHECK_ARG(out, "pg_eqn_create: out is NULL");
  *out = nullptr;
  PG_CHECK_ARG(m, "pg_eqn_create: NULL mesh");
  PG_CHECK_ARG(bc_type, "pg_eqn_create: bc_type is NULL");
  PG_CHECK_ARG(gamma_kind == PG_GAMMA_SCALAR || gamma_kind == PG_GAMMA_FACE,
               "pg_eqn_create: bad gamma_kind");
  const HostMesh &h = m->h;
  for (int64_t f = 0; f < h.n_faces; ++f)
    if (h.fr[f] < 0)
      PG_CHECK_ARG(bc_type[f] >= PG_BC_FIXED && bc_type[f] <= PG_BC_SYMMETRY,
                   "fv::laplacian: unrecognized or unspecified boundary type");
  auto *e = new (std::nothrow) pg_eqn();
  PG_CHECK_ARG(e, "pg_eqn_create: out of host memory");
  const int rc = eqn_fill(e, m, gamma_kind, bc_type, momentum, ib);
  if (rc) {
    delete e;
    return rc;
  }
  *out = e;
  return PG_OK;
}

extern "C" int pg_eqn_create_gcib(const pg_mesh *m, int gamma_kind,
                                  const int32_t *bc_type, int n_circles,
                                  const double *circles, int ib_bc,
                                  double ib_ref, pg_eqn **out) {
  PG_CHECK_ARG(out, "pg_eqn_create_gcib: out is NULL");
  *out = nullptr;
  PG_CHECK_ARG(m, "pg_eqn_create_gcib: NULL mesh");
  auto S = std::make_unique<GcibState>();
  S->ib_bc = ib_bc;
  S->ib_ref = ib_ref;
  GcibRows g;
  int rc = gcib_build(m, *S, n_circles, circles, g);
  if (rc) return rc;
  rc = eqn_create(m, gamma_kind, bc_type, false, out, &g);
  if (rc) return rc;
  (*out)->ib = std::move(S);
  return PG_OK;
}

extern "C" int pg_eqn_update_gcib(pg_eqn *e, int n_circles,
                                  const double *circles, double ib_ref,
                                  int *pattern_changed) {
  PG_CHECK_ARG(e && e->ib, "pg_eqn_update_gcib: not a ghost-cell IB equation");
  GcibState &S = *e->ib;
  const double old_ref = S.ib_ref;
  S.ib_ref = ib_ref;
  GcibRows g;
  bool changed = false;
  int rc = gcib_build(e->mesh, S, n_circles, circles, g, true, e->row_ptr.p,
                      e->col_ind.p, e->base_vals.p, e->base_rhs.p, &changed);
  if (rc) {
    S.ib_ref = old_ref;
    return rc;
  }
  if (changed) {
    const std::vector<int32_t> bc = e->bc_type;
    rc = eqn_fill(e, e->mesh, e->gamma_kind, bc.data(), false, &g);
    if (rc) return rc;
  }
  if (pattern_changed) *pattern_changed = changed ? 1 : 0;
  return PG_OK;
}

extern "C" int pg_eqn_cell_class(const pg_eqn *e, int32_t *cls) {
  PG_CHECK_ARG(e && cls, "pg_eqn_cell_class: NULL arg");
  for (int64_t c = 0; c < e->p.n; ++c)
    cls[c] = e->cell_class.empty() ? 0 : e->cell_class[c];
  return PG_OK;
}

extern "C" int pg_eqn_destroy(pg_eqn *e) {
  delete e;
  return PG_OK;
}

extern "C" int pg_eqn_sizes(const pg_eqn *e, int64_t *n_rows, int64_t *nnz) {
  PG_CHECK_ARG(e, "pg_eqn_sizes: NULL equation");
  if (n_rows) *n_rows = e->p.n;
  if (nnz) *nnz = e->p.nnz;
  return PG_OK;
}

extern "C" int pg_assemble_laplacian(pg_eqn *e, const double *gamma_face,
                                     double gamma_scalar,
                                     const double *bc_value,
                                     const double *u_face_xy, int ptr_kind) {
  PG_CHECK_ARG(e, "pg_assemble_laplacian: NULL equation");
  PG_CHECK_ARG(!e->momentum, "pg_assemble_laplacian: momentum equation");
  PG_CHECK_ARG((gamma_face != nullptr) == (e->gamma_kind == PG_GAMMA_FACE),
               "pg_assemble_laplacian: gamma_face must be given exactly for "
               "a PG_GAMMA_FACE equation");
  const HostMesh &h = e->mesh->h;
  const int64_t nf = h.n_faces;
  PG_CHECK_ARG(!e->any_fixed || bc_value,
               "pg_assemble_laplacian: bc_value needed for FIXED faces");
  const double *g = nullptr, *bv = nullptr, *u = nullptr;
  int rc = stage(gamma_face, nf, ptr_kind, e->stage_a, &g);
  if (!rc) rc = stage(bc_value, nf, ptr_kind, e->stage_b, &bv);
  if (!rc) rc = stage(u_face_xy, 2 * nf, ptr_kind, e->stage_c, &u);
  if (rc) return rc;
  cudaStream_t st = stream();
  if (e->has_base) {
    PG_CUDA(cudaMemcpyAsync(e->vals.p, e->base_vals.p, e->p.nnz * sizeof(double),
                            cudaMemcpyDeviceToDevice, st));
    PG_CUDA(cudaMemcpyAsync(e->rhs.p, e->base_rhs.p, e->p.n * sizeof(double),
                            cudaMemcpyDeviceToDevice, st));
  } else {
    PG_CUDA(cudaMemsetAsync(e->vals.p, 0, e->p.nnz * sizeof(double), st));
    PG_CUDA(cudaMemsetAsync(e->rhs.p, 0, e->p.n * sizeof(double), st));
  }
  const auto &cp = e->p.color_ptr;
  const int nic = e->p.n_interior_colors;
  for (int c = 0; c + 1 < (int)cp.size(); ++c) {
    const int off = cp[c], cnt = cp[c + 1] - cp[c];
    if (c < nic)
      launch_assemble_interior(cnt, off, e->cface.p, e->cl.p, e->cr.p,
                               e->cdot_l.p, e->cdot_r.p, e->cmsq.p,
                               e->slot_lr.p, e->slot_rl.p, e->diag_l.p,
                               e->diag_r.p, e->csfl_x.p, e->csfl_y.p,
                               e->csfr_x.p, e->csfr_y.p, g, gamma_scalar, u,
                               e->vals.p, e->rhs.p, st);
    else
      launch_assemble_boundary(cnt, off, e->cface.p, e->cl.p, e->cbc.p,
                               e->cdot_l.p, e->cmsq.p, e->diag_l.p,
                               e->csfl_x.p, e->csfl_y.p, g, gamma_scalar, bv,
                               u, e->vals.p, e->rhs.p, st);
  }
  PG_CUDA(cudaGetLastError());
  ++e->version;
  return PG_OK;
}

extern "C" int pg_eqn_device_values(const pg_eqn *e, double **vals,
                                    double **rhs) {
  PG_CHECK_ARG(e, "pg_eqn_device_values: NULL equation");
  if (vals) *vals = e->vals.p;
  if (rhs) *rhs = e->rhs.p;
  return PG_OK;
}

extern "C" int pg_eqn_export(const pg_eqn *e, int32_t *row_ptr,
                             int32_t *col_ind, double *vals, double *rhs) {
  PG_CHECK_ARG(e, "pg_eqn_export: NULL equation");
  if (e->has_base && (row_ptr || col_ind || vals)) {
    // A ghost-cell IB equation is CrsEquation::operator+ of the Laplacian and
    // the IB rows (CrsEquation.cpp:185-229), which leaves out every entry of
    // either operand that is exactly zero.  The device matrix keeps those
    // slots (the same operator); the exported CSR drops them.
    const int64_t n = e->p.n, nnz = e->p.nnz;
    std::vector<double> hv(nnz);
    PG_CUDA(copy_out(hv.data(), e->vals.p, nnz * sizeof(double), PG_HOST));
    PG_CUDA(cudaStreamSynchronize(stream()));
    int64_t k = 0;
    if (row_ptr) row_ptr[0] = 0;
    for (int64_t r = 0; r < n; ++r) {
      for (int32_t j = e->p.row_ptr[r]; j < e->p.row_ptr[r + 1]; ++j) {
        if (hv[j] == 0.) continue;
        if (col_ind) col_ind[k] = e->p.col_ind[j];
        if (vals) vals[k] = hv[j];
        ++k;
      }
      if (row_ptr) row_ptr[r + 1] = (int32_t)k;
    }
    row_ptr = nullptr;
    col_ind = nullptr;
    vals = nullptr;
  }
  if (row_ptr) std::copy(e->p.row_ptr.begin(), e->p.row_ptr.end(), row_ptr);
  if (col_ind) std::copy(e->p.col_ind.begin(), e->p.col_ind.end(), col_ind);
  if (vals) PG_CUDA(copy_out(vals, e->vals.p, e->p.nnz * sizeof(double), PG_HOST));
  if (rhs)
    PG_CUDA(copy_out(rhs, e->rhs.p,
                     (e->momentum ? 2 : 1) * e->p.n * sizeof(double), PG_HOST));
  PG_CUDA(cudaStreamSynchronize(stream()));
  return PG_OK;
}

// the diagonal a_ii of every row (the slot of e->diag; 0 where a row has
// none), device kernel
__global__ void k_eqn_diagonal(int n, const int32_t *__restrict__ diag,
                               const double *__restrict__ vals,
                               double *__restrict__ out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += gridDim.x * blockDim.x)
    out[i] = diag[i] >= 0 ? vals[diag[i]] : 0.;
}

extern "C" int pg_eqn_diagonal(const pg_eqn *e, double *diag, int ptr_kind) {
  PG_CHECK_ARG(e && diag, "pg_eqn_diagonal: NULL arg");
  PG_CHECK_ARG(e->diag.p, "pg_eqn_diagonal: equation has no diagonal map");
  const int n = (int)e->p.n;
  cudaStream_t st = stream();
  double *dst = diag;
  pg::DevBuf<double> tmp;
  if (ptr_kind != PG_DEVICE) {
    PG_CUDA(tmp.reserve(n));
    dst = tmp.p;
  }
  if (n > 0) {
    k_eqn_diagonal<<<(n + 255) / 256 < 2432 ? (n + 255) / 256 : 2432, 256, 0,
                     st>>>(n, e->diag.p, e->vals.p, dst);
    count_launches(1);
    PG_CUDA(cudaGetLastError());
  }
  if (ptr_kind != PG_DEVICE)
    PG_CUDA(copy_out(diag, dst, n * sizeof(double), PG_HOST));
  PG_CUDA(cudaStreamSynchronize(st));
  return PG_OK;
}

extern "C" int pg_assemble_momentum(pg_eqn *e, double dt, double nu,
                                    double theta, const double *u_old_cell,
                                    const double *u_face, int ptr_kind) {
  PG_CHECK_ARG(e && e->momentum, "pg_assemble_momentum: not a momentum equation");
  PG_CHECK_ARG(u_old_cell && u_face, "pg_assemble_momentum: NULL velocity");
  PG_CHECK_ARG(dt > 0., "pg_assemble_momentum: dt must be positive");
  const HostMesh &h = e->mesh->h;
  const double *u0 = nullptr, *uf = nullptr;
  int rc = stage(u_old_cell, 2 * h.n_cells, ptr_kind, e->stage_a, &u0);
  if (!rc) rc = stage(u_face, 2 * h.n_faces, ptr_kind, e->stage_c, &uf);
  if (rc) return rc;
  cudaStream_t st = stream();
  const int n = (int)e->p.n;
  PG_CUDA(cudaMemsetAsync(e->vals.p, 0, e->p.nnz * sizeof(double), st));
  launch_momentum_init(n, e->diag.p, e->mesh->d.vol.p, dt, u0, e->vals.p,
                       e->rhs.p, st);
  const auto &cp = e->p.color_ptr;
  const int nic = e->p.n_interior_colors;
  for (int c = 0; c + 1 < (int)cp.size(); ++c) {
    const int off = cp[c], cnt = cp[c + 1] - cp[c];
    if (c < nic)
      launch_momentum_interior(cnt, off, e->cface.p, e->cl.p, e->cr.p,
                               e->cdot_l.p, e->cdot_r.p, e->cmsq.p,
                               e->slot_lr.p, e->slot_rl.p, e->diag_l.p,
                               e->diag_r.p, e->csfl_x.p, e->csfl_y.p,
                               e->csfr_x.p, e->csfr_y.p, nu, theta, u0, uf, n,
                               e->vals.p, e->rhs.p, st);
    else
      launch_momentum_boundary(cnt, off, e->cface.p, e->cl.p, e->cbc.p,
                               e->cdot_l.p, e->cmsq.p, e->diag_l.p,
                               e->csfl_x.p, e->csfl_y.p, nu, theta, u0, uf, n,
                               e->vals.p, e->rhs.p, st);
  }
  PG_CUDA(cudaGetLastError());
  ++e->version;
  return PG_OK;
}

// ------------------------------------------------------------ field ops
extern "C" int pg_interpolate_faces(const pg_mesh *m, const double *cell_vals,
                                    double *face_vals, int ptr_kind) {
  PG_CHECK_ARG(m && cell_vals && face_vals, "pg_interpolate_faces: NULL arg");
  const HostMesh &h = m->h;
  DevBuf<double> gin, gout;
  const double *c = nullptr;
  int rc = stage(cell_vals, h.n_cells, ptr_kind, gin, &c);
  if (rc) return rc;
  double *o = face_vals;
  if (ptr_kind != PG_DEVICE) {
    PG_CUDA(gout.reserve(h.n_faces));
    o = gout.p;
  }
  launch_interp_faces((int)h.n_faces, m->d.fl.p, m->d.fr.p, m->d.fw.p, c, o,
                      stream());
  PG_CUDA(cudaGetLastError());
  if (ptr_kind != PG_DEVICE) {
    PG_CUDA(copy_out(face_vals, o, h.n_faces * sizeof(double), PG_HOST));
    PG_CUDA(cudaStreamSynchronize(stream()));
  }
  return PG_OK;
}

extern "C" int pg_face_dt_over_rho(const pg_mesh *m, const double *gamma_cell,
                                   double rho1, double rho2, double dt,
                                   double *coeff_face, int ptr_kind) {
  PG_CHECK_ARG(m && gamma_cell && coeff_face, "pg_face_dt_over_rho: NULL arg");
  const HostMesh &h = m->h;
  DevBuf<double> gin, gout;
  const double *g = nullptr;
  int rc = stage(gamma_cell, h.n_cells, ptr_kind, gin, &g);
  if (rc) return rc;
  double *o = coeff_face;
  if (ptr_kind != PG_DEVICE) {
    PG_CUDA(gout.reserve(h.n_faces));
    o = gout.p;
  }
  launch_dt_over_rho((int)h.n_faces, m->d.fl.p, m->d.fr.p, m->d.fw.p, g,
                     rho1, rho2, dt, o, stream());
  PG_CUDA(cudaGetLastError());
  if (ptr_kind != PG_DEVICE) {
    PG_CUDA(copy_out(coeff_face, o, h.n_faces * sizeof(double), PG_HOST));
    PG_CUDA(cudaStreamSynchronize(stream()));
  }
  return PG_OK;
}

extern "C" int pg_gradient(const pg_mesh *m, const double *phi_cell,
                           const double *phi_face, double *grad_face,
                           double *grad_cell, int ptr_kind) {
  PG_CHECK_ARG(m && phi_cell && phi_face, "pg_gradient: NULL arg");
  const HostMesh &h = m->h;
  DevBuf<double> a, b, gf, gc;
  const double *pc = nullptr, *pf = nullptr;
  int rc = stage(phi_cell, h.n_cells, ptr_kind, a, &pc);
  if (!rc) rc = stage(phi_face, h.n_faces, ptr_kind, b, &pf);
  if (rc) return rc;
  double *of = grad_face, *oc = grad_cell;
  if (ptr_kind != PG_DEVICE || !of) {
    PG_CUDA(gf.reserve(2 * h.n_faces));
    of = gf.p;
  }
  if (ptr_kind != PG_DEVICE && oc) {
    PG_CUDA(gc.reserve(2 * h.n_cells));
    oc = gc.p;
  }
  launch_gradient((int)h.n_cells, (int)h.n_faces, m->d.fl.p, m->d.fr.p,
                  m->d.fcx.p, m->d.fcy.p, m->d.cx.p, m->d.cy.p,
                  m->d.link_ptr.p, m->d.link_face.p, nullptr, nullptr,
                  m->d.fnx.p, m->d.fny.p, pc, pf, of, oc, stream());
  PG_CUDA(cudaGetLastError());
  if (ptr_kind != PG_DEVICE) {
    if (grad_face)
      PG_CUDA(copy_out(grad_face, of, 2 * h.n_faces * sizeof(double), PG_HOST));
    if (grad_cell)
      PG_CUDA(copy_out(grad_cell, oc, 2 * h.n_cells * sizeof(double), PG_HOST));
  }
  PG_CUDA(cudaStreamSynchronize(stream()));
  return PG_OK;
}

extern "C" int pg_set_boundary_faces(const pg_mesh *m, const int32_t *bc_type,
                                     const double *phi_cell, double *phi_face,
                                     int ptr_kind) {
  PG_CHECK_ARG(m && bc_type && phi_cell && phi_face,
               "pg_set_boundary_faces: NULL arg");
  const HostMesh &h = m->h;
  const int64_t n = h.n_cells, nf = h.n_faces;
  DevBuf<int32_t> bcd;
  DevBuf<double> pc, pf;
  const int32_t *bc = bc_type;
  const double *c = phi_cell;
  double *f = phi_face;
  if (ptr_kind != PG_DEVICE) {
    PG_CUDA(bcd.upload(bc_type, nf));
    PG_CUDA(pc.upload(phi_cell, n));
    PG_CUDA(pf.upload(phi_face, nf));
    bc = bcd.p;
    c = pc.p;
    f = pf.p;
  }
  launch_set_boundary_faces((int)nf, m->d.fl.p, m->d.fr.p, bc, c, f, stream());
  PG_CUDA(cudaGetLastError());
  if (ptr_kind != PG_DEVICE)
    PG_CUDA(copy_out(phi_face, f, nf * sizeof(double), PG_HOST));
  PG_CUDA(cudaStreamSynchronize(stream()));
  return PG_OK;
}

extern "C" int pg_correct_velocity(const pg_mesh *m, double dt,
                                   const double *rho_cell,
                                   const double *rho_face,
                                   const double *grad_cell,
                                   const double *grad_face, double *u_cell,
                                   double *u_face, int ptr_kind) {
  PG_CHECK_ARG(m && grad_cell && grad_face && u_cell && u_face,
               "pg_correct_velocity: NULL arg");
  PG_CHECK_ARG((rho_cell == nullptr) == (rho_face == nullptr),
               "pg_correct_velocity: give both densities or neither");
  const HostMesh &h = m->h;
  const int64_t n = h.n_cells, nf = h.n_faces;
  DevBuf<double> a, b, c, d, e, f;
  const double *rc = nullptr, *rf = nullptr, *gc = nullptr, *gf = nullptr;
  int rcode = stage(rho_cell, n, ptr_kind, a, &rc);
  if (!rcode) rcode = stage(rho_face, nf, ptr_kind, b, &rf);
  if (!rcode) rcode = stage(grad_cell, 2 * n, ptr_kind, c, &gc);
  if (!rcode) rcode = stage(grad_face, 2 * nf, ptr_kind, d, &gf);
  if (rcode) return rcode;
  double *uc = u_cell, *uf = u_face;
  if (ptr_kind != PG_DEVICE) {
    PG_CUDA(e.upload(u_cell, 2 * n));
    PG_CUDA(f.upload(u_face, 2 * nf));
    uc = e.p;
    uf = f.p;
  }
  launch_correct_velocity((int)n, dt, rc, gc, uc, stream());
  launch_correct_velocity((int)nf, dt, rf, gf, uf, stream());
  PG_CUDA(cudaGetLastError());
  if (ptr_kind != PG_DEVICE) {
    PG_CUDA(copy_out(u_cell, uc, 2 * n * sizeof(double), PG_HOST));
    PG_CUDA(copy_out(u_face, uf, 2 * nf * sizeof(double), PG_HOST));
  }
  PG_CUDA(cudaStreamSynchronize(stream()));
  return PG_OK;
}
