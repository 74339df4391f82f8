// CPU oracle for the Phase pressure-solve path -- TEST INFRASTRUCTURE ONLY.
// Restates the reference algorithms in plain C++ (no Boost, Eigen or
// Trilinos).  Only the tests, bench.py's CPU baseline and smoke() use it, as
// the checker; the product library never links it.
// Compiled with -ffp-contract=off so that products and sums round exactly as
// the reference's x86 build does (no fused multiply-add).
#include "oracle.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <map>
#include <numeric>
#include <queue>
#include <utility>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

using Clock = std::chrono::steady_clock;
static double ms_since(Clock::time_point t0) {
  return std::chrono::duration<double, std::milli>(Clock::now() - t0).count();
}

struct V2 {
  double x, y;
};
static inline double dot(V2 a, V2 b) { return a.x * b.x + a.y * b.y; }
static inline double mag_sqr(V2 a) { return a.x * a.x + a.y * a.y; }
static inline V2 sub(V2 a, V2 b) { return {a.x - b.x, a.y - b.y}; }

}  // namespace

struct or_mesh {
  std::vector<V2> nodes;
  std::vector<V2> centroid;
  std::vector<double> volume;
  // faces, in creation order (FiniteVolumeGrid2D::createCell)
  std::vector<int32_t> fl, fr, fln, frn;
  std::vector<V2> fc, fn;
  // per-cell link lists: interior links (face, cell) and boundary links
  // (face), each in face-id order (FiniteVolumeGrid2D::init :405-419)
  std::vector<std::vector<std::pair<int32_t, int32_t>>> nb;
  std::vector<std::vector<int32_t>> bd;
  // Node::cells(): the cells of each node in creation order; cell nodes
  std::vector<std::vector<int32_t>> node_cells, cell_nodes;
  int64_t n_interior = 0, n_boundary = 0;
};

// Face::outwardNorm(point) (Face.cpp:48-50)
static inline V2 outward_norm(const or_mesh &m, int32_t f, V2 p) {
  V2 n = m.fn[f];
  return dot(sub(m.fc[f], p), n) > 0. ? n : V2{-n.x, -n.y};
}

extern "C" or_mesh *or_mesh_create(const double *nodes_xy, int64_t n_nodes,
                                   const int64_t *cptr, const int64_t *cind,
                                   int64_t n_cells) {
  auto *m = new or_mesh();
  m->nodes.resize(n_nodes);
  for (int64_t i = 0; i < n_nodes; ++i)
    m->nodes[i] = {nodes_xy[2 * i], nodes_xy[2 * i + 1]};

  m->centroid.resize(n_cells);
  m->volume.resize(n_cells);
  m->node_cells.resize(n_nodes);
  m->cell_nodes.resize(n_cells);
  std::map<std::pair<int64_t, int64_t>, int32_t> dir;  // faceDirectory_

  for (int64_t c = 0; c < n_cells; ++c) {
    const int64_t b = cptr[c], e = cptr[c + 1], k = e - b;
    // Cell::Cell (Cell.cpp:8-29): polygon area and centroid (shoelace form
    // of the polygon area/centroid integrals; orientation corrected so the
    // area is positive).
    double a2 = 0., sx = 0., sy = 0.;
    for (int64_t i = 0; i < k; ++i) {
      V2 p = m->nodes[cind[b + i]], q = m->nodes[cind[b + (i + 1) % k]];
      double cr = p.x * q.y - q.x * p.y;
      a2 += cr;
      sx += (p.x + q.x) * cr;
      sy += (p.y + q.y) * cr;
    }
    m->volume[c] = std::fabs(a2) / 2.;
    m->centroid[c] = {sx / (3. * a2), sy / (3. * a2)};

    // FiniteVolumeGrid2D::createCell (FiniteVolumeGrid2D.cpp:84-114)
    for (int64_t i = 0; i < k; ++i) {
      m->node_cells[cind[b + i]].push_back((int32_t)c);
      m->cell_nodes[c].push_back((int32_t)cind[b + i]);
    }
    for (int64_t i = 0; i < k; ++i) {
      int64_t n1 = cind[b + i], n2 = cind[b + (i + 1) % k];
      auto key = n1 < n2 ? std::make_pair(n1, n2) : std::make_pair(n2, n1);
      auto it = dir.find(key);
      if (it == dir.end()) {
        int32_t id = (int32_t)m->fl.size();
        dir.emplace(key, id);
        V2 ln = m->nodes[n1], rn = m->nodes[n2];
        // Face::Face (Face.cpp:9-18): centroid = 0.5*(l+r), normal =
        // normalVec(r - l) = (t.y, -t.x) (Vector2D.h:26)
        m->fc.push_back({0.5 * (ln.x + rn.x), 0.5 * (ln.y + rn.y)});
        V2 t = sub(rn, ln);
        m->fn.push_back({t.y, -t.x});
        m->fl.push_back((int32_t)c);
        m->fr.push_back(-1);
        m->fln.push_back((int32_t)n1);
        m->frn.push_back((int32_t)n2);
      } else {
        m->fr[it->second] = (int32_t)c;
      }
    }
  }

  // FiniteVolumeGrid2D::init (:405-419): links in face-id order
  m->nb.resize(n_cells);
  m->bd.resize(n_cells);
  for (int32_t f = 0; f < (int32_t)m->fl.size(); ++f) {
    if (m->fr[f] < 0) {
      m->bd[m->fl[f]].push_back(f);
      ++m->n_boundary;
    } else {
      m->nb[m->fl[f]].push_back({f, m->fr[f]});
      m->nb[m->fr[f]].push_back({f, m->fl[f]});
      ++m->n_interior;
    }
  }
  return m;
}

extern "C" void or_mesh_destroy(or_mesh *m) { delete m; }

extern "C" void or_mesh_sizes(const or_mesh *m, int64_t *n_cells,
                              int64_t *n_faces, int64_t *n_interior,
                              int64_t *n_boundary) {
  *n_cells = (int64_t)m->centroid.size();
  *n_faces = (int64_t)m->fl.size();
  *n_interior = m->n_interior;
  *n_boundary = m->n_boundary;
}

extern "C" void or_mesh_cells(const or_mesh *m, double *cx, double *cy,
                              double *vol) {
  for (size_t c = 0; c < m->centroid.size(); ++c) {
    cx[c] = m->centroid[c].x;
    cy[c] = m->centroid[c].y;
    vol[c] = m->volume[c];
  }
}

extern "C" void or_mesh_faces(const or_mesh *m, int32_t *lcell,
                              int32_t *rcell, int32_t *lnode, int32_t *rnode,
                              double *fx, double *fy, double *nx, double *ny) {
  for (size_t f = 0; f < m->fl.size(); ++f) {
    lcell[f] = m->fl[f];
    rcell[f] = m->fr[f];
    lnode[f] = m->fln[f];
    rnode[f] = m->frn[f];
    fx[f] = m->fc[f].x;
    fy[f] = m->fc[f].y;
    nx[f] = m->fn[f].x;
    ny[f] = m->fn[f].y;
  }
}

extern "C" int64_t or_mesh_nlinks(const or_mesh *m) {
  return 2 * m->n_interior + m->n_boundary;
}

extern "C" void or_mesh_links(const or_mesh *m, int64_t *link_ptr,
                              int32_t *link_face, int32_t *link_cell) {
  int64_t k = 0;
  link_ptr[0] = 0;
  for (size_t c = 0; c < m->nb.size(); ++c) {
    for (auto &l : m->nb[c]) {
      link_face[k] = l.first;
      link_cell[k++] = l.second;
    }
    for (int32_t f : m->bd[c]) {
      link_face[k] = f;
      link_cell[k++] = -1;
    }
    link_ptr[c + 1] = k;
  }
}

// FiniteVolumeField::interpolateFaces(DISTANCE) (FiniteVolumeField.tpp
// :130-162) with Face::distanceWeight (Face.cpp:60-64), then
// setBoundaryFaces for NORMAL_GRADIENT patches (:165-183).
extern "C" void or_interpolate_faces(const or_mesh *m, const double *cv,
                                     double *fv) {
  for (size_t f = 0; f < m->fl.size(); ++f) {
    int32_t l = m->fl[f], r = m->fr[f];
    if (r < 0) {
      fv[f] = cv[l];
      continue;
    }
    V2 dr = sub(m->fc[f], m->centroid[r]);
    V2 dl = sub(m->fc[f], m->centroid[l]);
    double l1 = std::sqrt(dr.x * dr.x + dr.y * dr.y);
    double l2 = std::sqrt(dl.x * dl.x + dl.y * dl.y);
    double g = l1 / (l1 + l2);
    fv[f] = g * cv[l] + (1. - g) * cv[r];
  }
}

extern "C" void or_dt_over_rho_faces(const or_mesh *m, const double *gf,
                                     double rho1, double rho2, double dt,
                                     double *out) {
  for (size_t f = 0; f < m->fl.size(); ++f) {
    double g = std::min(std::max(gf[f], 0.), 1.);
    double rho = rho1 + g * (rho2 - rho1);
    out[f] = dt / rho;
  }
}

// ---------------------------------------------------------------------------
// CrsEquation semantics (CrsEquation.cpp:9-14 ctor with nnz=5 placeholder
// slots per row, :113-131 addCoeff).  Each row keeps its slots in a vector;
// an addCoeff that finds no free slot appends at the end of the row, which
// is where the reference inserts (colInd_.insert at rowPtr_[row+1]).
struct or_eqn {
  std::vector<std::vector<std::pair<int32_t, double>>> rows;
  std::vector<double> rhs;
};

static void add_coeff(or_eqn &e, int32_t row, int32_t col, double val) {
  auto &r = e.rows[row];
  for (auto &s : r) {
    if (s.first == col) {
      s.second += val;
      return;
    } else if (s.first == -1) {
      s.first = col;
      s.second = val;
      return;
    }
  }
  r.push_back({col, val});
}

// fv::laplacian over the cells with mask[c] != 0 (all when mask is NULL)
static or_eqn *laplacian_rows(const or_mesh *m, const double *gamma_face,
                              double gamma_scalar, const int32_t *bc_type,
                              const double *bc_value, const double *u_face_xy,
                              const uint8_t *mask) {
  const int64_t n = (int64_t)m->centroid.size();
  auto *e = new or_eqn();
  e->rows.assign(n, std::vector<std::pair<int32_t, double>>(5, {-1, 0.}));
  e->rhs.assign(n, 0.);

  for (int32_t c = 0; c < (int32_t)n; ++c) {
    if (mask && !mask[c]) continue;
    const V2 pc = m->centroid[c];
    for (auto &l : m->nb[c]) {
      const int32_t f = l.first, nbc = l.second;
      V2 rc = sub(m->centroid[nbc], pc);     // InteriorLink rCellVec
      V2 sf = outward_norm(*m, f, pc);       // InteriorLink outwardNorm
      if (gamma_face) {
        // Laplacian.h:139-142: diag first, then neighbour
        double coeff = gamma_face[f] * dot(rc, sf) / mag_sqr(rc);
        add_coeff(*e, c, c, -coeff);
        add_coeff(*e, c, nbc, coeff);
      } else {
        // Laplacian.h:55-58: neighbour first, then diag
        double coeff = gamma_scalar * dot(rc, sf) / mag_sqr(rc);
        add_coeff(*e, c, nbc, coeff);
        add_coeff(*e, c, c, -coeff);
      }
    }
    for (int32_t f : m->bd[c]) {
      V2 rf = sub(m->fc[f], pc);             // BoundaryLink rFaceVec
      V2 sf = outward_norm(*m, f, pc);
      double g = gamma_face ? gamma_face[f] : gamma_scalar;
      double coeff = g * dot(rf, sf) / mag_sqr(rf);
      switch (bc_type[f]) {
      case OR_FIXED:
        add_coeff(*e, c, c, -coeff);
        e->rhs[c] += coeff * bc_value[f];
        break;
      default:  // NORMAL_GRADIENT / SYMMETRY: no contribution
        break;
      }
    }
  }

  if (u_face_xy) {
    // src::div(u) (Source.cpp:5-21), then operator==(Vector) -> rhs_ -= divU
    // (CrsEquation.cpp:282-285,309-311)
    for (int32_t c = 0; c < (int32_t)n; ++c) {
      if (mask && !mask[c]) continue;
      const V2 pc = m->centroid[c];
      double d = 0.;
      for (auto &l : m->nb[c]) {
        int32_t f = l.first;
        V2 u{u_face_xy[2 * f], u_face_xy[2 * f + 1]};
        d += dot(u, outward_norm(*m, f, pc));
      }
      for (int32_t f : m->bd[c]) {
        V2 u{u_face_xy[2 * f], u_face_xy[2 * f + 1]};
        d += dot(u, outward_norm(*m, f, pc));
      }
      e->rhs[c] -= d;
    }
  }
  return e;
}

extern "C" or_eqn *or_laplacian(const or_mesh *m, const double *gamma_face,
                                double gamma_scalar, const int32_t *bc_type,
                                const double *bc_value,
                                const double *u_face_xy) {
  return laplacian_rows(m, gamma_face, gamma_scalar, bc_type, bc_value,
                        u_face_xy, nullptr);
}

extern "C" void or_eqn_destroy(or_eqn *e) { delete e; }

extern "C" void or_eqn_sizes(const or_eqn *e, int64_t *n, int64_t *n_slots,
                             int64_t *nnz) {
  *n = (int64_t)e->rows.size();
  int64_t s = 0, u = 0;
  for (auto &r : e->rows) {
    s += (int64_t)r.size();
    for (auto &p : r) u += p.first >= 0;
  }
  *n_slots = s;
  *nnz = u;
}

extern "C" void or_eqn_export_slots(const or_eqn *e, int32_t *row_ptr,
                                    int32_t *col_ind, double *vals,
                                    double *rhs) {
  int64_t k = 0;
  row_ptr[0] = 0;
  for (size_t i = 0; i < e->rows.size(); ++i) {
    for (auto &p : e->rows[i]) {
      col_ind[k] = p.first;
      vals[k++] = p.second;
    }
    row_ptr[i + 1] = (int32_t)k;
    rhs[i] = e->rhs[i];
  }
}

extern "C" void or_eqn_export_csr(const or_eqn *e, int32_t *row_ptr,
                                  int32_t *col_ind, double *vals,
                                  double *rhs) {
  int64_t k = 0;
  row_ptr[0] = 0;
  for (size_t i = 0; i < e->rows.size(); ++i) {
    for (auto &p : e->rows[i]) {
      if (p.first < 0) continue;
      col_ind[k] = p.first;
      vals[k++] = p.second;
    }
    row_ptr[i + 1] = (int32_t)k;
    rhs[i] = e->rhs[i];
  }
}

// ScalarGradient::computeFaces (ScalarGradient.cpp:34-47) and
// compute(FACE_TO_CELL) (:49-74)
extern "C" void or_gradient(const or_mesh *m, const double *phi,
                            const double *phi_face, double *gf,
                            double *gc) {
  const size_t nf = m->fl.size();
  for (size_t f = 0; f < nf; ++f) {
    int32_t l = m->fl[f], r = m->fr[f];
    V2 d;
    double dphi;
    if (r >= 0) {
      d = sub(m->centroid[r], m->centroid[l]);
      dphi = phi[r] - phi[l];
    } else {
      d = sub(m->fc[f], m->centroid[l]);
      dphi = phi_face[f] - phi[l];
    }
    double ms = mag_sqr(d);
    gf[2 * f] = dphi * d.x / ms;
    gf[2 * f + 1] = dphi * d.y / ms;
  }
  for (size_t c = 0; c < m->centroid.size(); ++c) {
    V2 sum{0., 0.}, tmp{0., 0.};
    auto acc = [&](int32_t f) {
      V2 sf = outward_norm(*m, f, m->centroid[c]);
      sf = {std::fabs(sf.x), std::fabs(sf.y)};
      tmp.x += gf[2 * f] * sf.x;
      tmp.y += gf[2 * f + 1] * sf.y;
      sum.x += sf.x;
      sum.y += sf.y;
    };
    for (auto &l : m->nb[c]) acc(l.first);
    for (int32_t f : m->bd[c]) acc(f);
    gc[2 * c] = tmp.x / sum.x;
    gc[2 * c + 1] = tmp.y / sum.y;
  }
}

// ---------------------------------------------------------------------------
// Sparse kernels and Krylov solver

namespace {

struct Csr {
  int64_t n;
  const int32_t *rp;
  const int32_t *ci;
  const double *v;
};

static void spmv(const Csr &A, const double *x, double *y) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < A.n; ++i) {
    double s = 0.;
    for (int32_t j = A.rp[i]; j < A.rp[i + 1]; ++j) s += A.v[j] * x[A.ci[j]];
    y[i] = s;
  }
}

// Dot product with a fixed summation order for a given thread count: each
// thread sums a contiguous chunk and the partials are added in thread order
// (an OpenMP reduction combines partials in an unspecified order, and the
// one-level BiCGStab is sensitive enough to those last bits to change its
// iteration count from run to run).
static double vdot(int64_t n, const double *a, const double *b) {
  std::vector<double> part(omp_get_max_threads(), 0.);
#pragma omp parallel
  {
    const int t = omp_get_thread_num(), nt = omp_get_num_threads();
    const int64_t lo = n * t / nt, hi = n * (t + 1) / nt;
    double s = 0.;
    for (int64_t i = lo; i < hi; ++i) s += a[i] * b[i];
    part[t] = s;
  }
  double s = 0.;
  for (double q : part) s += q;
  return s;
}

// Incomplete LU with zero fill, row-wise IKJ form (Saad, Iterative Methods
// for Sparse Linear Systems, 2nd ed., Alg. 10.4), restricted to the diagonal
// blocks of a row partition (Ifpack2 additive Schwarz, overlap 0, with a
// RILUK(0) subdomain solver).  Columns of each row are visited in increasing
// order; entries coupling two subdomains are excluded (stored as 0).
struct Ilu0 {
  int64_t n = 0;
  const int32_t *rp = nullptr, *ci = nullptr;
  std::vector<double> lu;
  std::vector<int32_t> diag;         // position of the diagonal per row
  std::vector<std::vector<int32_t>> order;  // per row: entry positions by col
  std::vector<std::vector<int32_t>> groups; // rows of each subdomain, sorted
  int status = 0;

  void build(const Csr &A, const int32_t *part, int n_parts) {
    n = A.n;
    rp = A.rp;
    ci = A.ci;
    lu.assign(A.v, A.v + A.rp[A.n]);
    diag.assign(n, -1);
    order.assign(n, {});
    for (int64_t i = 0; i < n; ++i) {
      auto &o = order[i];
      for (int32_t j = rp[i]; j < rp[i + 1]; ++j) {
        if (part && part[ci[j]] != part[i]) {
          lu[j] = 0.;
          continue;
        }
        o.push_back(j);
        if (ci[j] == i) diag[i] = j;
      }
      std::sort(o.begin(), o.end(),
                [&](int32_t a, int32_t b) { return ci[a] < ci[b]; });
    }
    if (part) {
      groups.assign(n_parts, {});
      for (int64_t i = 0; i < n; ++i) groups[part[i]].push_back((int32_t)i);
    } else {
      groups.assign(1, {});
      groups[0].resize(n);
      std::iota(groups[0].begin(), groups[0].end(), 0);
    }
    int bad = 0;
#pragma omp parallel
    {
      std::vector<int32_t> pos(n, -1);
#pragma omp for schedule(dynamic, 1) reduction(+ : bad)
      for (int64_t g = 0; g < (int64_t)groups.size(); ++g) {
        for (int32_t i : groups[g]) {
          for (int32_t j : order[i]) pos[ci[j]] = j;
          for (int32_t j : order[i]) {
            int32_t k = ci[j];
            if (k >= i) break;
            int32_t dk = diag[k];
            if (dk < 0 || lu[dk] == 0.) {
              ++bad;
              continue;
            }
            double lik = lu[j] / lu[dk];
            lu[j] = lik;
            for (int32_t jj : order[k]) {
              int32_t c = ci[jj];
              if (c <= k) continue;
              int32_t p = pos[c];
              if (p >= 0) lu[p] -= lik * lu[jj];
            }
          }
          for (int32_t j : order[i]) pos[ci[j]] = -1;
          if (diag[i] < 0 || lu[diag[i]] == 0. || !std::isfinite(lu[diag[i]]))
            ++bad;
        }
      }
    }
    status = bad ? 2 : 0;
  }

  void apply(const double *r, double *z) const {
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t g = 0; g < (int64_t)groups.size(); ++g) {
      const auto &rows = groups[g];
      for (int32_t i : rows) {
        double s = r[i];
        for (int32_t j : order[i]) {
          int32_t c = ci[j];
          if (c >= i) break;
          s -= lu[j] * z[c];
        }
        z[i] = s;
      }
      for (auto it = rows.rbegin(); it != rows.rend(); ++it) {
        int32_t i = *it;
        double s = z[i];
        for (auto jt = order[i].rbegin(); jt != order[i].rend(); ++jt) {
          int32_t c = ci[*jt];
          if (c <= i) break;
          s -= lu[*jt] * z[c];
        }
        z[i] = s / lu[diag[i]];
      }
    }
  }
};

// ILU(k) by levels of fill (Saad, Iterative Methods for Sparse Linear
// Systems, 2nd ed., sec. 10.3.3; Ifpack2 RILUK with "fact: iluk
// level-of-fill" k) on the diagonal blocks of a row partition: rows of a
// subdomain in increasing index, A's entries at level 0, a fill entry
// (i, j) at level lev(i,m) + lev(m,j) + 1 for m < i in row i and j > m in
// row m, kept when at most k; then the IKJ elimination on that pattern.
struct IluK {
  int64_t n = 0;
  std::vector<int64_t> rp, diag;
  std::vector<int32_t> ci;
  std::vector<double> v;
  std::vector<std::vector<int32_t>> groups;
  int status = 0;

  void build(const Csr &A, const int32_t *part, int n_parts, int p) {
    n = A.n;
    if (part) {
      groups.assign(n_parts, {});
      for (int64_t i = 0; i < n; ++i) groups[part[i]].push_back((int32_t)i);
    } else {
      groups.assign(1, {});
      for (int64_t i = 0; i < n; ++i) groups[0].push_back((int32_t)i);
    }
    // symbolic, per subdomain in row order; rows[i] = (column, level)
    std::vector<std::vector<std::pair<int32_t, int32_t>>> rows(n);
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t gi = 0; gi < (int64_t)groups.size(); ++gi) {
      std::map<int32_t, int32_t> lev;
      for (int32_t i : groups[gi]) {
        lev.clear();
        lev[i] = 0;
        for (int32_t j = A.rp[i]; j < A.rp[i + 1]; ++j)
          if (!part || part[A.ci[j]] == part[i]) lev[A.ci[j]] = 0;
        // keys inserted below are larger than the current one, so the
        // walk visits every lower entry, fill included, in increasing order
        for (auto it = lev.begin(); it != lev.end() && it->first < i; ++it) {
          const int32_t lim = it->second;
          for (const auto &e : rows[it->first]) {
            if (e.first <= it->first) continue;
            const int32_t lnew = lim + e.second + 1;
            if (lnew > p) continue;
            auto f = lev.find(e.first);
            if (f == lev.end()) lev.emplace(e.first, lnew);
            else if (lnew < f->second) f->second = lnew;
          }
        }
        rows[i].assign(lev.begin(), lev.end());
      }
    }
    rp.assign(n + 1, 0);
    for (int64_t i = 0; i < n; ++i) rp[i + 1] = rp[i] + (int64_t)rows[i].size();
    ci.resize(rp[n]);
    v.assign(rp[n], 0.);
    diag.assign(n, -1);
    for (int64_t i = 0; i < n; ++i) {
      for (size_t q = 0; q < rows[i].size(); ++q) {
        ci[rp[i] + q] = rows[i][q].first;
        if (rows[i][q].first == i) diag[i] = rp[i] + (int64_t)q;
      }
      for (int32_t j = A.rp[i]; j < A.rp[i + 1]; ++j) {
        if (part && part[A.ci[j]] != part[i]) continue;
        const auto b = ci.begin() + rp[i], e = ci.begin() + rp[i + 1];
        v[std::lower_bound(b, e, A.ci[j]) - ci.begin()] += A.v[j];
      }
    }
    // numeric IKJ on the pattern
    int bad = 0;
#pragma omp parallel reduction(+ : bad)
    {
      std::vector<int64_t> pos(n, -1);
#pragma omp for schedule(dynamic, 1)
      for (int64_t gi = 0; gi < (int64_t)groups.size(); ++gi) {
        for (int32_t i : groups[gi]) {
          for (int64_t j = rp[i]; j < rp[i + 1]; ++j) pos[ci[j]] = j;
          for (int64_t j = rp[i]; j < rp[i + 1] && ci[j] < i; ++j) {
            const int32_t m = ci[j];
            const double umm = v[diag[m]];
            if (umm == 0.) {
              ++bad;
              continue;
            }
            const double l = v[j] / umm;
            v[j] = l;
            for (int64_t q = diag[m] + 1; q < rp[m + 1]; ++q) {
              const int64_t pq = pos[ci[q]];
              if (pq >= 0) v[pq] -= l * v[q];
            }
          }
          for (int64_t j = rp[i]; j < rp[i + 1]; ++j) pos[ci[j]] = -1;
          if (v[diag[i]] == 0. || !std::isfinite(v[diag[i]])) ++bad;
        }
      }
    }
    status = bad ? 2 : 0;
  }

  void apply(const double *r, double *z) const {
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t g = 0; g < (int64_t)groups.size(); ++g) {
      const auto &gr = groups[g];
      for (int32_t i : gr) {
        double s = r[i];
        for (int64_t j = rp[i]; j < diag[i]; ++j) s -= v[j] * z[ci[j]];
        z[i] = s;
      }
      for (auto it = gr.rbegin(); it != gr.rend(); ++it) {
        const int32_t i = *it;
        double s = z[i];
        for (int64_t j = diag[i] + 1; j < rp[i + 1]; ++j) s -= v[j] * z[ci[j]];
        z[i] = s / v[diag[i]];
      }
    }
  }
};

// ILUT(p, tau): dual-threshold incomplete LU (Saad, "ILUT: a dual threshold
// incomplete LU factorization", Numer. Linear Algebra Appl. 1 (1994);
// Iterative Methods for Sparse Linear Systems, Alg. 10.6).  Row i is
// eliminated in a dense work row; multipliers and the final row are dropped
// below tau * ||a_i||_2, and at most p entries are kept in each of the L and
// U parts of the row (the diagonal is always kept).
struct Ilut {
  int64_t n = 0;
  std::vector<int64_t> lp, up;
  std::vector<int32_t> lc, uc;  // U rows store the diagonal first
  std::vector<double> lv, uv;
  int status = 0;

  void build(const Csr &A, double tau, int p) {
    n = A.n;
    lp.assign(1, 0);
    up.assign(1, 0);
    lc.clear(); uc.clear(); lv.clear(); uv.clear();
    std::vector<double> w(n, 0.);
    std::vector<char> in(n, 0);
    std::vector<int32_t> nzl, nzu;
    for (int64_t i = 0; i < n; ++i) {
      double nrm = 0.;
      nzl.clear();
      nzu.clear();
      bool has_diag = false;
      for (int32_t j = A.rp[i]; j < A.rp[i + 1]; ++j) {
        int32_t c = A.ci[j];
        nrm += A.v[j] * A.v[j];
        if (!in[c]) {
          in[c] = 1;
          (c < i ? nzl : nzu).push_back(c);
        }
        w[c] += A.v[j];
        if (c == i) has_diag = true;
      }
      if (!has_diag) {
        in[i] = 1;
        nzu.push_back((int32_t)i);
      }
      nrm = std::sqrt(nrm);
      const double tol = tau * nrm;
      // eliminate lower entries in increasing column order (min-heap)
      std::priority_queue<int32_t, std::vector<int32_t>, std::greater<int32_t>>
          heap(nzl.begin(), nzl.end());
      std::vector<int32_t> kept_l;
      while (!heap.empty()) {
        int32_t k = heap.top();
        heap.pop();
        double wk = w[k] / uv[up[k]];
        if (std::fabs(wk) < tol) {
          w[k] = 0.;
          continue;
        }
        w[k] = wk;
        kept_l.push_back(k);
        for (int64_t jj = up[k] + 1; jj < up[k + 1]; ++jj) {
          int32_t c = uc[jj];
          if (!in[c]) {
            in[c] = 1;
            if (c < i) {
              nzl.push_back(c);
              heap.push(c);
            } else {
              nzu.push_back(c);
            }
          }
          w[c] -= wk * uv[jj];
        }
      }
      // keep the p largest L multipliers
      std::sort(kept_l.begin(), kept_l.end(), [&](int32_t a, int32_t b) {
        return std::fabs(w[a]) > std::fabs(w[b]);
      });
      if ((int)kept_l.size() > p) kept_l.resize(p);
      std::sort(kept_l.begin(), kept_l.end());
      for (int32_t k : kept_l) {
        lc.push_back(k);
        lv.push_back(w[k]);
      }
      lp.push_back((int64_t)lc.size());
      // U part: drop small, keep p largest off-diagonals
      std::vector<int32_t> ku;
      for (int32_t c : nzu)
        if (c != i && std::fabs(w[c]) >= tol) ku.push_back(c);
      std::sort(ku.begin(), ku.end(), [&](int32_t a, int32_t b) {
        return std::fabs(w[a]) > std::fabs(w[b]);
      });
      if ((int)ku.size() > p) ku.resize(p);
      std::sort(ku.begin(), ku.end());
      double d = w[i];
      if (d == 0.) d = (tol > 0. ? tol : 1e-4);  // zero pivot replacement
      if (!std::isfinite(d)) status = 3;
      uc.push_back((int32_t)i);
      uv.push_back(d);
      for (int32_t c : ku) {
        uc.push_back(c);
        uv.push_back(w[c]);
      }
      up.push_back((int64_t)uc.size());
      for (int32_t c : nzl) { w[c] = 0.; in[c] = 0; }
      for (int32_t c : nzu) { w[c] = 0.; in[c] = 0; }
    }
  }

  void apply(const double *r, double *z) const {
    for (int64_t i = 0; i < n; ++i) {
      double s = r[i];
      for (int64_t j = lp[i]; j < lp[i + 1]; ++j) s -= lv[j] * z[lc[j]];
      z[i] = s;
    }
    for (int64_t i = n - 1; i >= 0; --i) {
      double s = z[i];
      for (int64_t j = up[i] + 1; j < up[i + 1]; ++j) s -= uv[j] * z[uc[j]];
      z[i] = s / uv[up[i]];
    }
  }
};

// Two-level coarse correction on the subdomain-constant vectors (the
// device solver's preconditioner, restated for an algorithm-matched CPU
// baseline; Nicolaides 1987, Tang, Nabben, Vuik & Erlangga 2009): A_c =
// Z^T A Z summed in FP64, factored by dense LU with partial pivoting
// (rows parallel over threads); a pivot below 1e-14 of the largest entry
// drops its coarse unknown (a singular, all-Neumann A_c).
struct Coarse {
  int K = 0;
  std::vector<double> lu;     // K x K, row-major, L unit-lower and U
  std::vector<int> piv;       // row permutation
  std::vector<char> dead;     // dropped unknowns
  const int32_t *part = nullptr;

  void build(const Csr &A, const int32_t *p, int k) {
    K = k;
    part = p;
    lu.assign((size_t)K * K, 0.);
    for (int64_t i = 0; i < A.n; ++i)
      for (int32_t j = A.rp[i]; j < A.rp[i + 1]; ++j)
        lu[(size_t)part[i] * K + part[A.ci[j]]] += A.v[j];
    double amax = 0.;
    for (double v : lu) amax = std::max(amax, std::fabs(v));
    piv.resize(K);
    dead.assign(K, 0);
    for (int c = 0; c < K; ++c) {
      int pr = c;
      for (int r = c + 1; r < K; ++r)
        if (std::fabs(lu[(size_t)r * K + c]) > std::fabs(lu[(size_t)pr * K + c])) pr = r;
      piv[c] = pr;
      if (pr != c)
        for (int j = 0; j < K; ++j) std::swap(lu[(size_t)c * K + j], lu[(size_t)pr * K + j]);
      const double d = lu[(size_t)c * K + c];
      if (std::fabs(d) <= 1e-14 * amax) {
        dead[c] = 1;
        continue;
      }
#pragma omp parallel for schedule(static)
      for (int r = c + 1; r < K; ++r) {
        double *row = &lu[(size_t)r * K];
        const double l = row[c] / d;
        row[c] = l;
        if (l != 0.)
          for (int j = c + 1; j < K; ++j) row[j] -= l * lu[(size_t)c * K + j];
      }
    }
    invert();
  }
  // y = A_c^-1 s with the LU factors (s overwritten)
  void lu_solve(std::vector<double> &s, std::vector<double> &y) const {
    for (int c = 0; c < K; ++c) std::swap(s[c], s[piv[c]]);
    for (int r = 0; r < K; ++r) {
      double acc = s[r];
      for (int j = 0; j < r; ++j) acc -= lu[(size_t)r * K + j] * s[j];
      s[r] = acc;
    }
    y.assign(K, 0.);
    for (int r = K - 1; r >= 0; --r) {
      if (dead[r]) continue;
      double acc = s[r];
      for (int j = r + 1; j < K; ++j) acc -= lu[(size_t)r * K + j] * y[j];
      y[r] = acc / lu[(size_t)r * K + r];
    }
  }
  // the explicit inverse (as the device applies it): column c solved from
  // the unit vector e_c, columns in parallel
  std::vector<double> inv;
  void invert() {
    inv.assign((size_t)K * K, 0.);
#pragma omp parallel
    {
      std::vector<double> e, y;
#pragma omp for schedule(dynamic, 8)
      for (int c = 0; c < K; ++c) {
        e.assign(K, 0.);
        e[c] = 1.;
        lu_solve(e, y);
        for (int r = 0; r < K; ++r) inv[(size_t)r * K + c] = y[r];
      }
    }
  }
  // y = A_c^-1 s (rows in parallel)
  void solve(std::vector<double> &s, std::vector<double> &y) const {
    y.assign(K, 0.);
#pragma omp parallel for schedule(static)
    for (int r = 0; r < K; ++r) {
      double acc = 0.;
      const double *row = &inv[(size_t)r * K];
      for (int c = 0; c < K; ++c) acc += row[c] * s[c];
      y[r] = acc;
    }
  }
  // Z^T r: subdomain sums in row order
  void sums(int64_t n, const double *r, std::vector<double> &s) const {
    s.assign(K, 0.);
    for (int64_t i = 0; i < n; ++i) s[part[i]] += r[i];
  }
};

struct Precond {
  int kind = OR_PREC_NONE;
  Ilu0 ilu0;
  IluK iluk;
  int fill = 0;
  Ilut ilut;
  std::vector<double> dinv;
  int status = 0;
  int coarse = 0;
  Coarse cs;
  const Csr *A = nullptr;
  mutable std::vector<double> s_, y_, t_;

  void build(const Csr &Am, const or_solver_cfg &cfg) {
    A = &Am;
    const Csr &A = Am;
    coarse = cfg.part && cfg.n_parts > 1 ? cfg.coarse : 0;
    if (coarse) cs.build(A, cfg.part, cfg.n_parts);
    kind = cfg.precond;
    fill = kind == OR_PREC_ILU0 ? cfg.ilu_fill : 0;
    if (kind == OR_PREC_ILU0 && fill > 0) {
      iluk.build(A, cfg.part, cfg.n_parts, fill);
      status = iluk.status;
    } else if (kind == OR_PREC_ILU0) {
      ilu0.build(A, cfg.part, cfg.n_parts);
      status = ilu0.status;
    } else if (kind == OR_PREC_ILUT) {
      ilut.build(A, cfg.ilut_drop, cfg.ilut_fill);
      status = ilut.status;
    } else if (kind == OR_PREC_JACOBI) {
      dinv.assign(A.n, 1.);
      for (int64_t i = 0; i < A.n; ++i)
        for (int32_t j = A.rp[i]; j < A.rp[i + 1]; ++j)
          if (A.ci[j] == i && A.v[j] != 0.) dinv[i] = 1. / A.v[j];
    }
  }
  void apply(int64_t n, const double *r, double *z) const {
    if (coarse == 2) {  // A-DEF1: y = A_c^-1 Z^T r, z = B (r - A Z y) + Z y
      cs.sums(n, r, s_);
      cs.solve(s_, y_);
      t_.resize(n);
#pragma omp parallel for schedule(static)
      for (int64_t i = 0; i < n; ++i) {
        double acc = r[i];
        for (int32_t j = A->rp[i]; j < A->rp[i + 1]; ++j)
          acc -= A->v[j] * y_[cs.part[A->ci[j]]];
        t_[i] = acc;
      }
      apply_one(n, t_.data(), z);
#pragma omp parallel for schedule(static)
      for (int64_t i = 0; i < n; ++i) z[i] += y_[cs.part[i]];
      return;
    }
    apply_one(n, r, z);
    if (coarse == 1) {  // additive: z += Z A_c^-1 Z^T r
      cs.sums(n, r, s_);
      cs.solve(s_, y_);
#pragma omp parallel for schedule(static)
      for (int64_t i = 0; i < n; ++i) z[i] += y_[cs.part[i]];
    }
  }
  void apply_one(int64_t n, const double *r, double *z) const {
    switch (kind) {
    case OR_PREC_ILU0:
      if (fill > 0) iluk.apply(r, z);
      else ilu0.apply(r, z);
      break;
    case OR_PREC_ILUT: ilut.apply(r, z); break;
    case OR_PREC_JACOBI:
#pragma omp parallel for schedule(static)
      for (int64_t i = 0; i < n; ++i) z[i] = dinv[i] * r[i];
      break;
    default:
      std::memcpy(z, r, sizeof(double) * n);
    }
  }
};

// BiCGStab (van der Vorst, SIAM J. Sci. Stat. Comput. 13 (1992)) with right
// preconditioning: A M^-1 y = b, x = M^-1 y.  The stop test is on the
// recursively updated residual, confirmed with a true residual b - A x; if
// the true residual has drifted above tol the iteration restarts from it.
// hist (optional) records ||r_k||/||b|| per iteration.
static int bicgstab(const Csr &A, const double *b, double *x,
                    const or_solver_cfg &cfg, or_solver_stats *st,
                    double *hist, int stop_on_tol) {
  const int64_t n = A.n;
  auto t_setup = Clock::now();
  Precond M;
  M.build(A, cfg);
  double setup_ms = ms_since(t_setup);
  auto t0 = Clock::now();

  std::vector<double> r(n), rh(n), p(n, 0.), v(n, 0.), ph(n), s(n), sh(n),
      t(n);
  if (!cfg.use_guess) std::fill(x, x + n, 0.);
  const double bn = std::sqrt(vdot(n, b, b));
  auto true_residual = [&]() {
    spmv(A, x, r.data());
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) r[i] = b[i] - r[i];
    return std::sqrt(vdot(n, r.data(), r.data()));
  };
  int status = 1, it = 0;
  double rn = true_residual();
  if (hist) hist[0] = bn > 0 ? rn / bn : 0.;
  if (bn == 0.) {
    std::fill(x, x + n, 0.);
    rn = 0.;
    status = 0;
  } else if (rn / bn <= cfg.tol && stop_on_tol) {
    status = 0;
  } else if (M.status) {
    status = M.status;
  } else {
    double rho_old = 1., alpha = 1., omega = 1.;
    rh = r;
    int restarts = 0;
    while (it < cfg.max_iters) {
      double rho = vdot(n, rh.data(), r.data());
      if (rho == 0.) { status = 2; break; }
      double beta = (rho / rho_old) * (alpha / omega);
#pragma omp parallel for schedule(static)
      for (int64_t i = 0; i < n; ++i) p[i] = r[i] + beta * (p[i] - omega * v[i]);
      M.apply(n, p.data(), ph.data());
      spmv(A, ph.data(), v.data());
      double rv = vdot(n, rh.data(), v.data());
      if (rv == 0.) { status = 2; break; }
      alpha = rho / rv;
#pragma omp parallel for schedule(static)
      for (int64_t i = 0; i < n; ++i) s[i] = r[i] - alpha * v[i];
      M.apply(n, s.data(), sh.data());
      spmv(A, sh.data(), t.data());
      double tt = vdot(n, t.data(), t.data());
      double ts = vdot(n, t.data(), s.data());
      omega = tt > 0. ? ts / tt : 0.;
#pragma omp parallel for schedule(static)
      for (int64_t i = 0; i < n; ++i) {
        x[i] += alpha * ph[i] + omega * sh[i];
        r[i] = s[i] - omega * t[i];
      }
      rho_old = rho;
      ++it;
      rn = std::sqrt(vdot(n, r.data(), r.data()));
      if (hist) hist[it] = rn / bn;
      if (!std::isfinite(rn)) { status = 3; break; }
      if (stop_on_tol && rn / bn <= cfg.tol) {
        rn = true_residual();
        if (rn / bn <= cfg.tol) { status = 0; break; }
        if (++restarts > 20) { status = 2; break; }
        rh = r;
        std::fill(p.begin(), p.end(), 0.);
        std::fill(v.begin(), v.end(), 0.);
        rho_old = alpha = omega = 1.;
      }
      if (omega == 0.) { status = 2; break; }
    }
  }
  double ms = ms_since(t0);
  if (st) {
    rn = true_residual();
    st->iters = it;
    st->status = status;
    st->rel_residual = bn > 0 ? rn / bn : 0.;
    st->ms = ms;
    st->setup_ms = setup_ms;
  }
  if (hist && !st) hist[cfg.max_iters + 1] = ms, hist[cfg.max_iters + 2] = setup_ms;
  return it;
}

// TFQMR (Freund 1993; Saad, Iterative Methods for Sparse Linear Systems,
// 2nd ed., Alg. 7.8) on A M^-1, x advanced by M^-1 d; one iteration is two
// half-steps.  Converged when sqrt(m+1) tau reaches the tolerance and the
// true residual confirms it; a failed confirmation or a breakdown restarts
// from the current x.
static int tfqmr(const Csr &A, const double *b, double *x,
                 const or_solver_cfg &cfg, or_solver_stats *st) {
  const int64_t n = A.n;
  auto t_setup = Clock::now();
  Precond M;
  M.build(A, cfg);
  const double setup_ms = ms_since(t_setup);
  auto t0 = Clock::now();
  if (!cfg.use_guess) std::fill(x, x + n, 0.);
  std::vector<double> w(n), u(n), uh(n), Bu(n), u1(n), uh1(n), Bu1(n), v(n),
      dh(n), rs(n), tmp(n);
  const double bn = std::sqrt(vdot(n, b, b));
  auto true_res = [&](std::vector<double> &r) {
    spmv(A, x, r.data());
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) r[i] = b[i] - r[i];
    return std::sqrt(vdot(n, r.data(), r.data()));
  };
  auto axpy = [&](double *out, double a, const double *p, double c,
                  const double *q) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) out[i] = a * p[i] + c * q[i];
  };
  int status = 1, it = 0, restarts = 0;
  double rn = 0.;
  if (bn == 0.) {
    std::fill(x, x + n, 0.);
    status = 0;
  } else if (M.status) {
    status = M.status;
  } else {
    for (;;) {
      rn = true_res(w);
      if (!std::isfinite(rn)) { status = 3; break; }
      if (rn / bn <= cfg.tol) { status = 0; break; }
      if (it >= cfg.max_iters) { status = 1; break; }
      u = w;
      rs = w;
      std::fill(dh.begin(), dh.end(), 0.);
      M.apply(n, u.data(), uh.data());
      spmv(A, uh.data(), Bu.data());
      v = Bu;
      double tau = rn, theta = 0., eta = 0., rho = rn * rn, alpha = 0.;
      int m = 0;
      bool restart = false, done = false;
      auto half = [&](const double *uhm, const double *Bum) {
        axpy(w.data(), 1., w.data(), -alpha, Bum);
        axpy(dh.data(), 1., uhm, theta * theta / alpha * eta, dh.data());
        theta = std::sqrt(vdot(n, w.data(), w.data())) / tau;
        const double c = 1. / std::sqrt(1. + theta * theta);
        tau = tau * theta * c;
        eta = c * c * alpha;
        axpy(x, 1., x, eta, dh.data());
        ++m;
        done = tau * std::sqrt((double)m + 1.) <= cfg.tol * bn;
      };
      while (it < cfg.max_iters) {
        const double sigma = vdot(n, v.data(), rs.data());
        if (sigma == 0. || rho == 0. || !std::isfinite(sigma)) {
          restart = true;
          break;
        }
        alpha = rho / sigma;
        axpy(u1.data(), 1., u.data(), -alpha, v.data());
        half(uh.data(), Bu.data());
        M.apply(n, u1.data(), uh1.data());
        spmv(A, uh1.data(), Bu1.data());
        if (!done) half(uh1.data(), Bu1.data());
        ++it;
        if (done) break;
        const double rho_new = vdot(n, w.data(), rs.data());
        const double beta = rho_new / rho;
        rho = rho_new;
        axpy(u.data(), 1., w.data(), beta, u1.data());
        M.apply(n, u.data(), uh.data());
        spmv(A, uh.data(), tmp.data());
        axpy(v.data(), 1., Bu1.data(), beta, v.data());
        axpy(v.data(), 1., tmp.data(), beta, v.data());
        Bu = tmp;
      }
      if (restart && ++restarts > 50) { status = 2; break; }
    }
  }
  if (st) {
    rn = true_res(w);
    st->iters = it;
    st->status = status;
    st->rel_residual = bn > 0 ? rn / bn : 0.;
    st->ms = ms_since(t0);
    st->setup_ms = setup_ms;
  }
  return it;
}

// Restarted GMRES (Saad & Schultz 1986) on A M^-1 with modified
// Gram-Schmidt and Givens rotations; x += M^-1 (V y) at the end of each
// cycle; converged when the implicit residual |g_{j+1}| reaches the
// tolerance and the true residual confirms it.
static int gmres(const Csr &A, const double *b, double *x,
                 const or_solver_cfg &cfg, or_solver_stats *st) {
  const int64_t n = A.n;
  const int dim = cfg.krylov_dim > 0 ? cfg.krylov_dim : 300;
  auto t_setup = Clock::now();
  Precond M;
  M.build(A, cfg);
  const double setup_ms = ms_since(t_setup);
  auto t0 = Clock::now();
  if (!cfg.use_guess) std::fill(x, x + n, 0.);
  std::vector<double> r(n), z(n), w(n), V((size_t)(dim + 1) * n);
  std::vector<double> H((size_t)(dim + 1) * dim), cs(dim), sn(dim), g(dim + 1),
      y(dim);
  const double bn = std::sqrt(vdot(n, b, b));
  auto true_res = [&]() {
    spmv(A, x, r.data());
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) r[i] = b[i] - r[i];
    return std::sqrt(vdot(n, r.data(), r.data()));
  };
  int status = 1, it = 0;
  double rn = 0.;
  if (bn == 0.) {
    std::fill(x, x + n, 0.);
    status = 0;
  } else if (M.status) {
    status = M.status;
  } else {
    for (;;) {
      rn = true_res();
      if (!std::isfinite(rn)) { status = 3; break; }
      if (rn / bn <= cfg.tol) { status = 0; break; }
      if (it >= cfg.max_iters) { status = 1; break; }
      for (int64_t i = 0; i < n; ++i) V[i] = r[i] / rn;
      std::fill(g.begin(), g.end(), 0.);
      g[0] = rn;
      int j = 0;
      for (; j < dim && it < cfg.max_iters; ++j) {
        const double *vj = &V[(size_t)j * n];
        M.apply(n, vj, z.data());
        spmv(A, z.data(), w.data());
        for (int i = 0; i <= j; ++i) {
          const double *vi = &V[(size_t)i * n];
          const double hij = vdot(n, w.data(), vi);
          H[(size_t)i * dim + j] = hij;
#pragma omp parallel for schedule(static)
          for (int64_t k = 0; k < n; ++k) w[k] -= hij * vi[k];
        }
        const double hn = std::sqrt(vdot(n, w.data(), w.data()));
        ++it;
        if (hn > 0.)
          for (int64_t k = 0; k < n; ++k) V[(size_t)(j + 1) * n + k] = w[k] / hn;
        double hj1 = hn;
        for (int i = 0; i < j; ++i) {
          double &a0 = H[(size_t)i * dim + j], &a1 = H[(size_t)(i + 1) * dim + j];
          const double t = cs[i] * a0 + sn[i] * a1;
          a1 = -sn[i] * a0 + cs[i] * a1;
          a0 = t;
        }
        double &hjj = H[(size_t)j * dim + j];
        const double den = std::hypot(hjj, hj1);
        cs[j] = den > 0. ? hjj / den : 1.;
        sn[j] = den > 0. ? hj1 / den : 0.;
        hjj = den;
        g[j + 1] = -sn[j] * g[j];
        g[j] = cs[j] * g[j];
        if (std::fabs(g[j + 1]) <= cfg.tol * bn || den == 0.) {
          ++j;
          break;
        }
      }
      for (int i = j - 1; i >= 0; --i) {
        double acc = g[i];
        for (int k = i + 1; k < j; ++k) acc -= H[(size_t)i * dim + k] * y[k];
        const double hii = H[(size_t)i * dim + i];
        y[i] = hii != 0. ? acc / hii : 0.;
      }
      std::fill(w.begin(), w.end(), 0.);
      for (int i = 0; i < j; ++i)
        for (int64_t k = 0; k < n; ++k) w[k] += y[i] * V[(size_t)i * n + k];
      M.apply(n, w.data(), z.data());
      for (int64_t k = 0; k < n; ++k) x[k] += z[k];
    }
  }
  if (st) {
    rn = true_res();
    st->iters = it;
    st->status = status;
    st->rel_residual = bn > 0 ? rn / bn : 0.;
    st->ms = ms_since(t0);
    st->setup_ms = setup_ms;
  }
  return it;
}

struct ThreadScope {
  int saved = 0;
  explicit ThreadScope(int k) {
#ifdef _OPENMP
    saved = omp_get_max_threads();
    if (k > 0) omp_set_num_threads(k);
#endif
  }
  ~ThreadScope() {
#ifdef _OPENMP
    omp_set_num_threads(saved);
#endif
  }
};

}  // namespace

extern "C" int or_bicgstab(int64_t n, const int32_t *row_ptr,
                           const int32_t *col_ind, const double *vals,
                           const double *b, double *x,
                           const or_solver_cfg *cfg, or_solver_stats *stats) {
  ThreadScope ts(cfg->n_threads);
  Csr A{n, row_ptr, col_ind, vals};
  or_solver_stats st{};
  if (cfg->krylov == 1)
    tfqmr(A, b, x, *cfg, &st);
  else if (cfg->krylov == 2)
    gmres(A, b, x, *cfg, &st);
  else
    bicgstab(A, b, x, *cfg, &st, nullptr, 1);
  if (stats) *stats = st;
  return st.status;
}

extern "C" int or_bicgstab_history_x0(int64_t n, const int32_t *row_ptr,
                                      const int32_t *col_ind,
                                      const double *vals, const double *b,
                                      const double *x0,
                                      const or_solver_cfg *cfg, double *hist,
                                      double *ms_out, double *setup_ms_out) {
  ThreadScope ts(cfg->n_threads);
  Csr A{n, row_ptr, col_ind, vals};
  std::vector<double> x(n, 0.);
  if (x0) std::copy(x0, x0 + n, x.begin());
  or_solver_cfg c = *cfg;
  c.use_guess = x0 ? 1 : 0;
  std::vector<double> h(c.max_iters + 3, 0.);
  int it = bicgstab(A, b, x.data(), c, nullptr, h.data(), 0);
  for (int i = 0; i <= it; ++i) hist[i] = h[i];
  *ms_out = h[c.max_iters + 1];
  *setup_ms_out = h[c.max_iters + 2];
  return it;
}

extern "C" int or_bicgstab_history(int64_t n, const int32_t *row_ptr,
                                   const int32_t *col_ind, const double *vals,
                                   const double *b, const or_solver_cfg *cfg,
                                   double *hist, double *ms_out,
                                   double *setup_ms_out) {
  return or_bicgstab_history_x0(n, row_ptr, col_ind, vals, b, nullptr, cfg,
                                hist, ms_out, setup_ms_out);
}

extern "C" int or_iluk_apply(int64_t n, const int32_t *row_ptr,
                             const int32_t *col_ind, const double *vals,
                             const int32_t *part, int fill, const double *r,
                             double *z) {
  Csr A{n, row_ptr, col_ind, vals};
  int np = 0;
  if (part)
    for (int64_t i = 0; i < n; ++i) np = std::max(np, part[i] + 1);
  IluK f;
  f.build(A, part, np, fill);
  if (f.status) return f.status;
  f.apply(r, z);
  return 0;
}

extern "C" int or_ilu0(int64_t n, const int32_t *row_ptr,
                       const int32_t *col_ind, const double *vals,
                       const int32_t *part, double *out_vals) {
  Csr A{n, row_ptr, col_ind, vals};
  Ilu0 f;
  int np = 0;
  if (part)
    for (int64_t i = 0; i < n; ++i) np = std::max(np, part[i] + 1);
  f.build(A, part, np);
  std::copy(f.lu.begin(), f.lu.end(), out_vals);
  return f.status;
}

extern "C" void or_ilu0_apply(int64_t n, const int32_t *row_ptr,
                              const int32_t *col_ind, const double *lu_vals,
                              const int32_t *part, const double *r,
                              double *z) {
  // rebuild the row orders; the factor values are taken as given
  Csr A{n, row_ptr, col_ind, lu_vals};
  Ilu0 f;
  int np = 0;
  if (part)
    for (int64_t i = 0; i < n; ++i) np = std::max(np, part[i] + 1);
  f.n = n;
  f.rp = row_ptr;
  f.ci = col_ind;
  f.lu.assign(lu_vals, lu_vals + row_ptr[n]);
  f.diag.assign(n, -1);
  f.order.assign(n, {});
  for (int64_t i = 0; i < n; ++i) {
    for (int32_t j = row_ptr[i]; j < row_ptr[i + 1]; ++j) {
      if (part && part[col_ind[j]] != part[i]) continue;
      f.order[i].push_back(j);
      if (col_ind[j] == i) f.diag[i] = j;
    }
    std::sort(f.order[i].begin(), f.order[i].end(),
              [&](int32_t a, int32_t b) { return col_ind[a] < col_ind[b]; });
  }
  if (part) {
    f.groups.assign(np, {});
    for (int64_t i = 0; i < n; ++i) f.groups[part[i]].push_back((int32_t)i);
  } else {
    f.groups.assign(1, std::vector<int32_t>(n));
    std::iota(f.groups[0].begin(), f.groups[0].end(), 0);
  }
  (void)A;
  f.apply(r, z);
}

extern "C" void or_spmv(int64_t n, const int32_t *row_ptr,
                        const int32_t *col_ind, const double *vals,
                        const double *x, double *y) {
  Csr A{n, row_ptr, col_ind, vals};
  spmv(A, x, y);
}

// ---------------------------------------------------------------------------
// Momentum operator (config: lid-driven cavity SIMPLE predictor)

namespace {
// CrsEquation::operator+= / -= (CrsEquation.cpp:185-229, 231-275): rebuild
// each row from the entries of the left side that are non-zero and not
// placeholders, then add the right side's non-zero entries (summing into an
// existing column or appending).
static void crs_plus(or_eqn &a, const or_eqn &b, double sign) {
  for (size_t r = 0; r < a.rows.size(); ++r) {
    std::vector<std::pair<int32_t, double>> out;
    for (auto &e : a.rows[r])
      if (e.second != 0. && e.first >= 0) out.push_back(e);
    for (auto &e : b.rows[r]) {
      if (e.second == 0. || e.first < 0) continue;
      bool found = false;
      for (auto &o : out)
        if (o.first == e.first) {
          o.second += sign * e.second;
          found = true;
          break;
        }
      if (!found) out.push_back({e.first, sign * e.second});
    }
    a.rows[r] = std::move(out);
    a.rhs[r] += sign * b.rhs[r];
  }
}
}  // namespace

extern "C" or_eqn *or_momentum(const or_mesh *m, double dt, double nu,
                               double theta, const double *u0,
                               const double *uf, const int32_t *bc_type) {
  const int64_t n = (int64_t)m->centroid.size();
  auto fresh = [&]() {
    auto *e = new or_eqn();
    e->rows.assign(2 * n, std::vector<std::pair<int32_t, double>>(5, {-1, 0.}));
    e->rhs.assign(2 * n, 0.);
    return e;
  };
  // add to both components (FiniteVolumeEquation<Vector2D>::add, :17-30)
  auto add2 = [&](or_eqn &e, int32_t c, int32_t col, double v) {
    add_coeff(e, c, col, v);
    add_coeff(e, (int32_t)(n + c), (int32_t)(n + col), v);
  };
  // fv::ddt(field, dt) (TimeDerivative.h:38-48)
  or_eqn *ddt = fresh();
  for (int32_t c = 0; c < (int32_t)n; ++c) {
    const double v = m->volume[c];
    add2(*ddt, c, c, v / dt);
    ddt->rhs[c] += -v * u0[2 * c] / dt;
    ddt->rhs[n + c] += -v * u0[2 * c + 1] / dt;
  }
  // fv::div(u, phi, theta) (Divergence.h:8-53), old-time terms use u0 = u
  or_eqn *div = fresh();
  for (int32_t c = 0; c < (int32_t)n; ++c) {
    const V2 pc = m->centroid[c];
    for (auto &l : m->nb[c]) {
      const int32_t f = l.first, nbc = l.second;
      const V2 sf = outward_norm(*m, f, pc);
      const double flux = uf[2 * f] * sf.x + uf[2 * f + 1] * sf.y;
      add2(*div, c, c, theta * std::max(flux, 0.));
      add2(*div, c, nbc, theta * std::min(flux, 0.));
      const double f0 = flux;  // old flux: same face velocity
      div->rhs[c] += (1. - theta) * std::max(f0, 0.) * u0[2 * c];
      div->rhs[n + c] += (1. - theta) * std::max(f0, 0.) * u0[2 * c + 1];
      div->rhs[c] += (1. - theta) * std::min(f0, 0.) * u0[2 * nbc];
      div->rhs[n + c] += (1. - theta) * std::min(f0, 0.) * u0[2 * nbc + 1];
    }
    for (int32_t f : m->bd[c]) {
      const V2 sf = outward_norm(*m, f, pc);
      const double flux = uf[2 * f] * sf.x + uf[2 * f + 1] * sf.y;
      switch (bc_type[f]) {
      case OR_FIXED:
        div->rhs[c] += theta * flux * uf[2 * f];
        div->rhs[n + c] += theta * flux * uf[2 * f + 1];
        div->rhs[c] += (1. - theta) * flux * uf[2 * f];
        div->rhs[n + c] += (1. - theta) * flux * uf[2 * f + 1];
        break;
      case OR_NORMAL_GRADIENT:
        add2(*div, c, c, theta * flux);
        div->rhs[c] += (1. - theta) * flux * u0[2 * c];
        div->rhs[n + c] += (1. - theta) * flux * u0[2 * c + 1];
        break;
      default:
        break;
      }
    }
  }
  // fv::laplacian(gamma, phi, theta) (Laplacian.h:7-47), scalar gamma
  or_eqn *lap = fresh();
  for (int32_t c = 0; c < (int32_t)n; ++c) {
    const V2 pc = m->centroid[c];
    for (auto &l : m->nb[c]) {
      const int32_t f = l.first, nbc = l.second;
      const V2 rc = sub(m->centroid[nbc], pc);
      const double coeff = nu * dot(rc, outward_norm(*m, f, pc)) / mag_sqr(rc);
      add2(*lap, c, nbc, theta * coeff);
      add2(*lap, c, c, theta * -coeff);
      lap->rhs[c] += (1. - theta) * coeff * (u0[2 * nbc] - u0[2 * c]);
      lap->rhs[n + c] += (1. - theta) * coeff * (u0[2 * nbc + 1] - u0[2 * c + 1]);
    }
    for (int32_t f : m->bd[c]) {
      const V2 rf = sub(m->fc[f], pc);
      const double coeff = nu * dot(rf, outward_norm(*m, f, pc)) / mag_sqr(rf);
      if (bc_type[f] == OR_FIXED) {
        add2(*lap, c, c, theta * -coeff);
        lap->rhs[c] += theta * coeff * uf[2 * f];
        lap->rhs[n + c] += theta * coeff * uf[2 * f + 1];
        lap->rhs[c] += (1. - theta) * coeff * (uf[2 * f] - u0[2 * c]);
        lap->rhs[n + c] += (1. - theta) * coeff * (uf[2 * f + 1] - u0[2 * c + 1]);
      }
    }
  }
  // ddt + div == laplacian  ->  (ddt += div) -= laplacian
  crs_plus(*ddt, *div, 1.);
  crs_plus(*ddt, *lap, -1.);
  delete div;
  delete lap;
  return ddt;
}

// ---------------------------------------------------------------- GCIB
namespace {

// LU factorisation with partial pivoting followed by inversion, the
// algorithm of LAPACK dgetrf + dgetri that StaticMatrix::invert calls
// (src/Math/StaticMatrix.h:82-91); returns false for a singular matrix.
static bool invert4(const double (&a_in)[4][4], double (&inv)[4][4]) {
  double a[4][4];
  int piv[4];
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) a[i][j] = a_in[i][j];
  for (int k = 0; k < 4; ++k) {
    int p = k;
    for (int i = k + 1; i < 4; ++i)
      if (std::fabs(a[i][k]) > std::fabs(a[p][k])) p = i;
    piv[k] = p;
    if (a[p][k] == 0.) return false;
    if (p != k)
      for (int j = 0; j < 4; ++j) std::swap(a[k][j], a[p][j]);
    for (int i = k + 1; i < 4; ++i) {
      a[i][k] /= a[k][k];
      for (int j = k + 1; j < 4; ++j) a[i][j] -= a[i][k] * a[k][j];
    }
  }
  // solve A X = P^T I column by column: forward (unit L), backward (U)
  double e[4][4] = {{1, 0, 0, 0}, {0, 1, 0, 0}, {0, 0, 1, 0}, {0, 0, 0, 1}};
  for (int k = 0; k < 4; ++k)
    if (piv[k] != k)
      for (int j = 0; j < 4; ++j) std::swap(e[k][j], e[piv[k]][j]);
  for (int c = 0; c < 4; ++c) {
    double y[4];
    for (int i = 0; i < 4; ++i) {
      double s = e[i][c];
      for (int j = 0; j < i; ++j) s -= a[i][j] * y[j];
      y[i] = s;
    }
    for (int i = 3; i >= 0; --i) {
      double s = y[i];
      for (int j = i + 1; j < 4; ++j) s -= a[i][j] * inv[j][c];
      inv[i][c] = s / a[i][i];
    }
  }
  return true;
}

static inline V2 unit(V2 v) {
  const double m = std::sqrt(v.x * v.x + v.y * v.y);
  return {v.x / m, v.y / m};
}

}  // namespace

// Ghost-cell immersed-boundary pressure equation of FractionalStepGCIB
// (src/2D/Unstructured/Solvers/FractionalStepGCIB.cpp:44-46):
//   (fv::laplacian(gamma, p) + ib.bcs(p)) == src::div(u)
// with the cell classes of GhostCellImmersedBoundary::updateCells
// (GhostCellImmersedBoundary.cpp:12-30): a cell whose centroid is strictly
// inside a circle (Circle::isInside) is an IB cell when one of its
// cellLinks (face and node neighbours) is outside that circle
// (ImmersedBoundaryObject.tpp internalPerimeterCells, includeDiagonals),
// otherwise solid; the rest are fluid, and the Laplacian and the source
// run over the fluid cells only.  bcs(p) (GhostCellImmersedBoundary.cpp:
// 32-74) adds, per IB cell, the stencil of GhostCellImmersedBoundary
// BcStencil (GhostCellImmersedBoundaryBcStencil.cpp:3-69): bp = nearest
// point of the circle, ip = 2 bp - x_c, nw = unit(centre - bp), the four
// cells of the node nearest to ip (FiniteVolumeGrid2D::findNearestNode,
// Node::cells in creation order) and Ainv = inverse of the rows
// [x y, x, y, 1] of their centroids; NORMAL_GRADIENT
// (…NormalGradientBcStencil.cpp:17-40): [bp.y nx + bp.x ny, nx, ny, 0] Ainv
// if the IB cell is one of the four, else -[ip.x ip.y, ip.x, ip.y, 1] Ainv/l
// and 1/l on the cell itself (l = |ip - x_c|); FIXED (…FixedBcStencil.cpp:
// 17-22): [ip.x ip.y, ip.x, ip.y, 1] Ainv / 2 and 1/2 on the cell; source
// -ref.  Solid cells: identity row, source -ref (FIXED) or rhs 0.  The sum
// is CrsEquation::operator+ (crs_plus above).  circles[3k..3k+2] = cx, cy, r.
// Returns NULL when a stencil matrix is singular or a node has other than
// four cells.
extern "C" or_eqn *or_gcib_laplacian(const or_mesh *m, const double *gamma_face,
                                     double gamma_scalar,
                                     const int32_t *bc_type,
                                     const double *bc_value,
                                     const double *u_face_xy, int n_circles,
                                     const double *circles, int ib_bc,
                                     double ib_ref, int32_t *cell_class) {
  const int32_t n = (int32_t)m->centroid.size();
  std::vector<int32_t> cls(n, 0);  // 0 fluid, 1 IB, 2 solid
  std::vector<std::vector<int32_t>> ibc(n_circles);
  for (int k = 0; k < n_circles; ++k) {
    const V2 cc{circles[3 * k], circles[3 * k + 1]};
    const double r = circles[3 * k + 2];
    auto inside = [&](int32_t c) { return mag_sqr(sub(m->centroid[c], cc)) < r * r; };
    for (int32_t c = 0; c < n; ++c) {
      if (cls[c] != 0 || !inside(c)) continue;
      bool perimeter = false;
      for (int32_t nd : m->cell_nodes[c])
        for (int32_t o : m->node_cells[nd])
          if (o != c && !inside(o)) perimeter = true;
      cls[c] = perimeter ? 1 : 2;
      if (perimeter) ibc[k].push_back(c);
    }
  }
  std::vector<uint8_t> fluid(n);
  for (int32_t c = 0; c < n; ++c) fluid[c] = cls[c] == 0;
  or_eqn *lap = laplacian_rows(m, gamma_face, gamma_scalar, bc_type, bc_value,
                               u_face_xy, fluid.data());
  or_eqn bcs;
  bcs.rows.assign(n, std::vector<std::pair<int32_t, double>>(5, {-1, 0.}));
  bcs.rhs.assign(n, 0.);
  for (int k = 0; k < n_circles; ++k) {
    const V2 cc{circles[3 * k], circles[3 * k + 1]};
    const double r = circles[3 * k + 2];
    for (int32_t c : ibc[k]) {
      const V2 xc = m->centroid[c];
      const V2 u = unit(sub(xc, cc));
      const V2 bp{u.x * r + cc.x, u.y * r + cc.y};
      const V2 ip{2. * bp.x - xc.x, 2. * bp.y - xc.y};
      const V2 nw = unit(sub(cc, bp));
      // nearest node (first of equals in id order)
      int32_t best = -1;
      double bd = 0.;
      for (int32_t v = 0; v < (int32_t)m->nodes.size(); ++v) {
        const double d = mag_sqr(sub(m->nodes[v], ip));
        if (best < 0 || d < bd) { best = v; bd = d; }
      }
      const auto &st = m->node_cells[best];
      if (st.size() != 4) { delete lap; return nullptr; }
      double A[4][4], Ai[4][4];
      for (int i = 0; i < 4; ++i) {
        const V2 x = m->centroid[st[i]];
        A[i][0] = x.x * x.y; A[i][1] = x.x; A[i][2] = x.y; A[i][3] = 1.;
      }
      if (!invert4(A, Ai)) { delete lap; return nullptr; }
      auto rowvec = [&](const double (&w)[4], double (&out)[4]) {
        for (int j = 0; j < 4; ++j) {
          double s = 0.;
          for (int i = 0; i < 4; ++i) s += w[i] * Ai[i][j];
          out[j] = s;
        }
      };
      double co[4];
      if (ib_bc == OR_FIXED) {
        const double w[4] = {ip.x * ip.y, ip.x, ip.y, 1.};
        rowvec(w, co);
        for (int j = 0; j < 4; ++j) add_coeff(bcs, c, st[j], co[j] / 2.);
        add_coeff(bcs, c, c, 0.5);
      } else {
        bool in_st = false;
        for (int32_t o : st) in_st |= o == c;
        if (in_st) {
          const double w[4] = {bp.y * nw.x + bp.x * nw.y, nw.x, nw.y, 0.};
          rowvec(w, co);
          for (int j = 0; j < 4; ++j) add_coeff(bcs, c, st[j], co[j]);
        } else {
          const double l = std::sqrt(mag_sqr(sub(ip, xc)));
          const double w[4] = {ip.x * ip.y, ip.x, ip.y, 1.};
          rowvec(w, co);
          for (int j = 0; j < 4; ++j) add_coeff(bcs, c, st[j], -co[j] / l);
          add_coeff(bcs, c, c, 1. / l);
        }
      }
      bcs.rhs[c] += -ib_ref;
    }
  }
  for (int32_t c = 0; c < n; ++c) {
    if (cls[c] != 2) continue;
    add_coeff(bcs, c, c, 1.);
    if (ib_bc == OR_FIXED) bcs.rhs[c] += -ib_ref;
    else bcs.rhs[c] = 0.;
  }
  crs_plus(*lap, bcs, 1.);
  if (cell_class) std::copy(cls.begin(), cls.end(), cell_class);
  return lap;
}

// FiniteVolumeField::setBoundaryFaces (src/2D/Unstructured/FiniteVolume/
// Field/FiniteVolumeField.tpp:165-183): every face of a NORMAL_GRADIENT or
// SYMMETRY patch takes the value of its lCell; FIXED patches and interior
// faces are left as they are.
extern "C" void or_set_boundary_faces(const or_mesh *m, const int32_t *bc_type,
                                      const double *phi_cell,
                                      double *phi_face) {
  for (size_t f = 0; f < m->fl.size(); ++f)
    if (m->fr[f] < 0 && bc_type[f] != OR_FIXED)
      phi_face[f] = phi_cell[m->fl[f]];
}

// FractionalStep::correctVelocity (src/2D/Unstructured/Solvers/
// FractionalStep.cpp:109-117) and FractionalStepMultiphase::correctVelocity
// (FractionalStepMultiphase.cpp:165-173): u -= timeStep / rho * gradP on
// every cell and every face; rho NULL = 1.
extern "C" void or_correct_velocity(const or_mesh *m, double dt,
                                    const double *rho_cell,
                                    const double *rho_face,
                                    const double *grad_cell,
                                    const double *grad_face, double *u_cell,
                                    double *u_face) {
  const int64_t n = (int64_t)m->centroid.size(), nf = (int64_t)m->fl.size();
  for (int64_t c = 0; c < n; ++c) {
    const double k = rho_cell ? dt / rho_cell[c] : dt;
    u_cell[2 * c] -= k * grad_cell[2 * c];
    u_cell[2 * c + 1] -= k * grad_cell[2 * c + 1];
  }
  for (int64_t f = 0; f < nf; ++f) {
    const double k = rho_face ? dt / rho_face[f] : dt;
    u_face[2 * f] -= k * grad_face[2 * f];
    u_face[2 * f + 1] -= k * grad_face[2 * f + 1];
  }
}

// ------------------------------------------------------------ direct solve
// EigenSparseMatrixSolver (src/Math/EigenSparseMatrixSolver.cpp:17-64): the
// matrix of the entries with col >= 0 (repeated entries summed, as
// setFromTriplets), factorised with partial pivoting and solved.  Restated
// as a band LU: a reverse Cuthill-McKee ordering (Cuthill & McKee 1969,
// reversed as George 1971) of the symmetrised pattern, then Gaussian
// elimination with row partial pivoting inside the band (the storage
// scheme of LAPACK's dgbtrf: pivoting widens the upper band from ku to
// kl + ku).  Any stable LU gives the same x up to rounding, which is what
// the parity tests compare.  A pivot at most 1e-13 of its column's largest
// entry in A is replaced by that entry (a consistent singular system then
// gets one of its solutions).
namespace {

std::vector<int32_t> rcm_order(int64_t n, const std::vector<int64_t> &ap,
                               const std::vector<int32_t> &aj) {
  std::vector<int32_t> order;
  order.reserve(n);
  std::vector<char> done(n, 0);
  std::vector<int64_t> deg(n);
  for (int64_t i = 0; i < n; ++i) deg[i] = ap[i + 1] - ap[i];
  auto bfs = [&](int32_t s, std::vector<int32_t> &out) {
    std::vector<char> seen(n, 0);
    out.clear();
    out.push_back(s);
    seen[s] = 1;
    for (size_t h = 0; h < out.size(); ++h) {
      const int32_t u = out[h];
      std::vector<int32_t> nb;
      for (int64_t e = ap[u]; e < ap[u + 1]; ++e)
        if (!seen[aj[e]] && !done[aj[e]]) nb.push_back(aj[e]);
      std::sort(nb.begin(), nb.end(), [&](int32_t a, int32_t b) {
        return deg[a] < deg[b] || (deg[a] == deg[b] && a < b);
      });
      for (int32_t w : nb) {
        seen[w] = 1;
        out.push_back(w);
      }
    }
  };
  std::vector<int32_t> comp;
  for (int64_t s0 = 0; s0 < n; ++s0) {
    if (done[s0]) continue;
    // pseudo-peripheral start: the last vertex of a BFS from the
    // component's first vertex
    bfs((int32_t)s0, comp);
    bfs(comp.back(), comp);
    for (int32_t u : comp) done[u] = 1;
    order.insert(order.end(), comp.begin(), comp.end());
  }
  std::reverse(order.begin(), order.end());
  return order;
}

}  // namespace

extern "C" int or_sparse_lu_solve(int64_t n, const int32_t *row_ptr,
                                  const int32_t *col_ind, const double *vals,
                                  const double *b, double *x, int64_t *band,
                                  int *replaced) {
  // compact matrix, duplicates summed
  std::vector<std::map<int32_t, double>> rows(n);
  for (int64_t i = 0; i < n; ++i)
    for (int64_t k = row_ptr[i]; k < row_ptr[i + 1]; ++k)
      if (col_ind[k] >= 0) rows[i][col_ind[k]] += vals[k];
  std::vector<double> cmax(n, 0.);
  std::vector<int64_t> ap(n + 1, 0);
  std::vector<int32_t> aj;
  {
    std::vector<std::vector<int32_t>> adj(n);
    for (int64_t i = 0; i < n; ++i)
      for (auto &e : rows[i]) {
        cmax[e.first] = std::max(cmax[e.first], std::fabs(e.second));
        if (e.first != i) {
          adj[i].push_back(e.first);
          adj[e.first].push_back((int32_t)i);
        }
      }
    for (int64_t i = 0; i < n; ++i) {
      std::sort(adj[i].begin(), adj[i].end());
      adj[i].erase(std::unique(adj[i].begin(), adj[i].end()), adj[i].end());
      ap[i + 1] = ap[i] + (int64_t)adj[i].size();
      aj.insert(aj.end(), adj[i].begin(), adj[i].end());
    }
  }
  const std::vector<int32_t> order = rcm_order(n, ap, aj);  // new -> old
  std::vector<int32_t> inv(n);
  for (int64_t i = 0; i < n; ++i) inv[order[i]] = (int32_t)i;
  int64_t kl = 0, ku = 0;
  for (int64_t i = 0; i < n; ++i)
    for (auto &e : rows[i]) {
      const int64_t r = inv[i], c = inv[e.first];
      kl = std::max(kl, r - c);
      ku = std::max(ku, c - r);
    }
  const int64_t w = 2 * kl + ku + 1;  // row window: columns i-kl .. i+kl+ku
  std::vector<double> W((size_t)(n * w), 0.);
  auto at = [&](int64_t i, int64_t j) -> double & {
    return W[(size_t)(i * w + (j - i + kl))];
  };
  for (int64_t i = 0; i < n; ++i)
    for (auto &e : rows[i]) at(inv[i], inv[e.first]) = e.second;
  std::vector<int64_t> piv(n);
  int nrep = 0;
  for (int64_t c = 0; c < n; ++c) {
    const int64_t rlast = std::min(n - 1, c + kl);
    const int64_t jlast = std::min(n - 1, c + kl + ku);
    int64_t p = c;
    double best = std::fabs(at(c, c));
    for (int64_t r = c + 1; r <= rlast; ++r)
      if (std::fabs(at(r, c)) > best) {
        best = std::fabs(at(r, c));
        p = r;
      }
    piv[c] = p;
    if (p != c)
      for (int64_t j = c; j <= jlast; ++j) std::swap(at(c, j), at(p, j));
    const double cs = cmax[order[c]];
    if (std::fabs(at(c, c)) <= 1e-13 * cs || at(c, c) == 0.) {
      at(c, c) = cs > 0. ? cs : 1.;
      ++nrep;
    }
    const double d = at(c, c);
    for (int64_t r = c + 1; r <= rlast; ++r) {
      const double l = at(r, c) / d;
      at(r, c) = l;
      if (l != 0.)
        for (int64_t j = c + 1; j <= jlast; ++j) at(r, j) -= l * at(c, j);
    }
  }
  std::vector<double> y(n);
  for (int64_t i = 0; i < n; ++i) y[i] = b[order[i]];
  for (int64_t c = 0; c < n; ++c) {
    if (piv[c] != c) std::swap(y[c], y[piv[c]]);
    const double yc = y[c];
    const int64_t rlast = std::min(n - 1, c + kl);
    for (int64_t r = c + 1; r <= rlast; ++r) y[r] -= at(r, c) * yc;
  }
  for (int64_t c = n - 1; c >= 0; --c) {
    const int64_t jlast = std::min(n - 1, c + kl + ku);
    double s = y[c];
    for (int64_t j = c + 1; j <= jlast; ++j) s -= at(c, j) * y[j];
    y[c] = s / at(c, c);
  }
  for (int64_t i = 0; i < n; ++i) x[order[i]] = y[i];
  if (band) {
    band[0] = kl;
    band[1] = ku;
  }
  if (replaced) *replaced = nrep;
  return 0;
}
