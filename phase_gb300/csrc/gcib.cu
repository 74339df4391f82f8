// Ghost-cell immersed-boundary stencils built on the device.
//
// GhostCellImmersedBoundary::updateCells (src/2D/Unstructured/FiniteVolume/
// ImmersedBoundary/GhostCellImmersedBoundary.cpp:12-30) classifies the cells
// of every IB object, and the solvers with moving bodies call it after
// every position update (FractionalStepDFIB.cpp:29-31; a body moves by
// Motion::update, e.g. OscillatingMotion.cpp:12-24).
// GhostCellImmersedBoundary::bcs (:32-74) then builds each IB cell's row
// from its stencil (GhostCellImmersedBoundaryBcStencil.cpp:3-69: boundary
// point, image point, the four cells of the node nearest to the image point
// (FiniteVolumeGrid2D::findNearestNode, FiniteVolumeGrid2D.cpp:210-212) and
// the inverse of their bilinear matrix; FixedBcStencil.cpp:17-22,
// NormalGradientBcStencil.cpp:17-40).
//
// Kernels (one stream, the library's):
//   k_gcib_classify  one thread per cell: the first circle whose interior
//                    holds the centroid, then the perimeter test over the
//                    cells that share a node with the cell; IB cells are
//                    appended to a list (its order does not matter: every
//                    IB cell owns its row);
//   k_gcib_stencil   one thread per IB cell: boundary and image points,
//                    nearest node by a ring search of the bucket grid,
//                    Gauss-Jordan inverse of the 4x4 bilinear matrix,
//                    coefficients;
//   k_gcib_scatter   bodies moved with every cell keeping its class: the
//                    new IB rows are written into the equation's constant
//                    rows in place, or a flag says the pattern changed;
//   k_gcib_rhs       the constant rhs of the IB and solid rows.
// Geometry uses explicitly rounded operations (no fused multiply-add), so
// the classes and the stencil cells are those of an FP64 host computation
// without contraction.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <mutex>
#include <string>
#include <vector>

#include "internal.h"

namespace pg {
namespace {

__device__ __forceinline__ double sq2(double dx, double dy) {
  return __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
}

// Circle::isInside: |x - c|^2 < r^2
__device__ __forceinline__ bool in_circle(double x, double y,
                                          const double *c) {
  return sq2(__dsub_rn(x, c[0]), __dsub_rn(y, c[1])) < __dmul_rn(c[2], c[2]);
}

__global__ void k_gcib_classify(int n, const double *__restrict__ cx,
                                const double *__restrict__ cy, int nc,
                                const double *__restrict__ circ,
                                const int32_t *__restrict__ cptr,
                                const int32_t *__restrict__ cind,
                                const int32_t *__restrict__ nptr,
                                const int32_t *__restrict__ ncell,
                                const int32_t *__restrict__ old_cls,
                                int32_t *__restrict__ cls,
                                int2 *__restrict__ ib,
                                int32_t *__restrict__ counters) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  const double x = cx[c], y = cy[c];
  int k0 = -1;
  for (int k = 0; k < nc; ++k)
    if (in_circle(x, y, circ + 3 * k)) {
      k0 = k;
      break;
    }
  int cl = 0;
  if (k0 >= 0) {
    // internalPerimeterCells with diagonals: a cell sharing a node with c
    // lies outside this circle
    const double *cc = circ + 3 * k0;
    bool per = false;
    for (int q = cptr[c]; q < cptr[c + 1] && !per; ++q) {
      const int v = cind[q];
      for (int t = nptr[v]; t < nptr[v + 1]; ++t) {
        const int o = ncell[t];
        if (o != c && !in_circle(cx[o], cy[o], cc)) {
          per = true;
          break;
        }
      }
    }
    cl = per ? 1 : 2;
    if (per) ib[atomicAdd(&counters[0], 1)] = make_int2(c, k0);
  }
  cls[c] = cl;
  if (old_cls && old_cls[c] != cl) counters[3] = 1;
}

struct NodeGridDev {
  const int32_t *start, *items;
  const double *x, *y;
  double x0, y0, h;
  int nx, ny;
};

__device__ __forceinline__ int bucket_index(double v, double v0, double h,
                                            int nb) {
  double f = floor(__ddiv_rn(__dsub_rn(v, v0), h));
  f = fmin(fmax(f, 0.), (double)(nb - 1));
  return (int)f;
}

// The node nearest to (x, y): smallest squared distance, then smallest id
// (the first of equals in id order).  Buckets are searched in square rings
// around the query's bucket; a node outside the rings searched so far is
// more than (ring - 1) h away, so the search stops once the best distance
// is below that.
__device__ int nearest_node(const NodeGridDev &g, double x, double y) {
  const int ix = bucket_index(x, g.x0, g.h, g.nx);
  const int iy = bucket_index(y, g.y0, g.h, g.ny);
  int best = -1;
  double bd = 0.;
  const int max_ring = max(g.nx, g.ny);
  for (int ring = 0; ring <= max_ring; ++ring) {
    for (int dy = -ring; dy <= ring; ++dy) {
      const int by = iy + dy;
      if (by < 0 || by >= g.ny) continue;
      const int step = (ring == 0 || dy == -ring || dy == ring) ? 1 : 2 * ring;
      for (int dx = -ring; dx <= ring; dx += step) {
        const int bx = ix + dx;
        if (bx < 0 || bx >= g.nx) continue;
        const int64_t b = (int64_t)by * g.nx + bx;
        for (int k = g.start[b]; k < g.start[b + 1]; ++k) {
          const int v = g.items[k];
          const double d = sq2(__dsub_rn(g.x[v], x), __dsub_rn(g.y[v], y));
          if (best < 0 || d < bd || (d == bd && v < best)) {
            best = v;
            bd = d;
          }
        }
      }
    }
    if (best >= 0 && ring >= 1) {
      const double lim = (double)(ring - 1) * g.h;
      if (bd < lim * lim) break;
    }
  }
  return best;
}

// Inverse of a 4x4 matrix by Gauss-Jordan elimination with partial
// pivoting on [A | I]; false if a pivot is zero.
__device__ bool inverse4_dev(const double (&a)[4][4], double (&out)[4][4]) {
  double w[4][8];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) w[i][j] = j < 4 ? a[i][j] : (j - 4 == i ? 1. : 0.);
  for (int k = 0; k < 4; ++k) {
    int p = k;
    for (int i = k + 1; i < 4; ++i)
      if (fabs(w[i][k]) > fabs(w[p][k])) p = i;
    if (w[p][k] == 0.) return false;
    if (p != k)
      for (int j = 0; j < 8; ++j) {
        const double t = w[p][j];
        w[p][j] = w[k][j];
        w[k][j] = t;
      }
    const double piv = w[k][k];
    for (int j = 0; j < 8; ++j) w[k][j] = __ddiv_rn(w[k][j], piv);
    for (int i = 0; i < 4; ++i) {
      if (i == k) continue;
      const double f = w[i][k];
      for (int j = 0; j < 8; ++j)
        w[i][j] = __dsub_rn(w[i][j], __dmul_rn(f, w[k][j]));
    }
  }
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) out[i][j] = w[i][4 + j];
  return true;
}

__device__ __forceinline__ void fail(int32_t *counters, int code, int cell) {
  atomicCAS(&counters[1], 0, code);
  atomicMin(&counters[2], cell);
}

__global__ void k_gcib_stencil(int n_ib, const int2 *__restrict__ ib,
                               const double *__restrict__ circ, int ib_bc,
                               const double *__restrict__ cx,
                               const double *__restrict__ cy, NodeGridDev g,
                               const int32_t *__restrict__ nptr,
                               const int32_t *__restrict__ ncell,
                               GcibStencil *__restrict__ out,
                               int32_t *__restrict__ counters) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_ib) return;
  const int c = ib[i].x, k = ib[i].y;
  const double ccx = circ[3 * k], ccy = circ[3 * k + 1], r = circ[3 * k + 2];
  const double xc = cx[c], yc = cy[c];
  // boundary point bp = unit(x_c - centre) r + centre, image point
  // ip = 2 bp - x_c, wall normal nw = unit(centre - bp)
  const double dx = __dsub_rn(xc, ccx), dy = __dsub_rn(yc, ccy);
  const double dm = __dsqrt_rn(sq2(dx, dy));
  const double bpx = __dadd_rn(__dmul_rn(__ddiv_rn(dx, dm), r), ccx);
  const double bpy = __dadd_rn(__dmul_rn(__ddiv_rn(dy, dm), r), ccy);
  const double ipx = __dsub_rn(__dmul_rn(2., bpx), xc);
  const double ipy = __dsub_rn(__dmul_rn(2., bpy), yc);
  const double tx = __dsub_rn(ccx, bpx), ty = __dsub_rn(ccy, bpy);
  const double tm = __dsqrt_rn(sq2(tx, ty));
  const double nwx = __ddiv_rn(tx, tm), nwy = __ddiv_rn(ty, tm);
  GcibStencil s;
  s.cell = c;
  s.circle = k;
  s.has_self = 0;
  s.pad = 0;
  s.self = 0.;
  for (int j = 0; j < 4; ++j) {
    s.st[j] = c;
    s.co[j] = 0.;
  }
  const int node = nearest_node(g, ipx, ipy);
  if (node < 0 || nptr[node + 1] - nptr[node] != 4) {
    fail(counters, 1, c);
    out[i] = s;
    return;
  }
  double A[4][4], Ai[4][4];
  for (int j = 0; j < 4; ++j) {
    const int o = ncell[nptr[node] + j];
    s.st[j] = o;
    const double x = cx[o], y = cy[o];
    A[j][0] = __dmul_rn(x, y);
    A[j][1] = x;
    A[j][2] = y;
    A[j][3] = 1.;
  }
  if (!inverse4_dev(A, Ai)) {
    fail(counters, 2, c);
    out[i] = s;
    return;
  }
  double w[4];
  bool in_st = false;
  for (int j = 0; j < 4; ++j) in_st |= s.st[j] == c;
  const bool ng_self = ib_bc != PG_BC_FIXED && in_st;
  if (ng_self) {  // NormalGradientBcStencil, the IB cell among the four
    w[0] = __dadd_rn(__dmul_rn(bpy, nwx), __dmul_rn(bpx, nwy));
    w[1] = nwx;
    w[2] = nwy;
    w[3] = 0.;
  } else {
    w[0] = __dmul_rn(ipx, ipy);
    w[1] = ipx;
    w[2] = ipy;
    w[3] = 1.;
  }
  double co[4];
  for (int j = 0; j < 4; ++j) {
    double acc = __dmul_rn(w[0], Ai[0][j]);
    acc = __dadd_rn(acc, __dmul_rn(w[1], Ai[1][j]));
    acc = __dadd_rn(acc, __dmul_rn(w[2], Ai[2][j]));
    co[j] = __dadd_rn(acc, __dmul_rn(w[3], Ai[3][j]));
  }
  if (ib_bc == PG_BC_FIXED) {  // FixedBcStencil: (interp(ip) + phi_c) / 2
    for (int j = 0; j < 4; ++j) s.co[j] = __ddiv_rn(co[j], 2.);
    s.has_self = 1;
    s.self = 0.5;
  } else if (ng_self) {
    for (int j = 0; j < 4; ++j) s.co[j] = co[j];
  } else {  // (phi_c - interp(ip)) / l
    const double l = __dsqrt_rn(sq2(__dsub_rn(ipx, xc), __dsub_rn(ipy, yc)));
    for (int j = 0; j < 4; ++j) s.co[j] = __ddiv_rn(-co[j], l);
    s.has_self = 1;
    s.self = __ddiv_rn(1., l);
  }
  out[i] = s;
}

// Sums an IB stencil into its row entries (column order of first
// appearance, as CrsEquation::addCoeff accumulates); returns the count.
__device__ __forceinline__ int merge_row(const GcibStencil &s, int (&cols)[5],
                                         double (&vals)[5]) {
  int m = 0;
  auto add = [&](int col, double v) {
    for (int q = 0; q < m; ++q)
      if (cols[q] == col) {
        vals[q] = __dadd_rn(vals[q], v);
        return;
      }
    cols[m] = col;
    vals[m] = v;
    ++m;
  };
  for (int j = 0; j < 4; ++j) add(s.st[j], s.co[j]);
  if (s.has_self) add(s.cell, s.self);
  return m;
}

__global__ void k_gcib_scatter(int n_ib, const GcibStencil *__restrict__ st,
                               const int32_t *__restrict__ rp,
                               const int32_t *__restrict__ ci,
                               double *__restrict__ base_vals,
                               int32_t *__restrict__ counters) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  // a failed stencil leaves the equation as it was
  if (i >= n_ib || counters[1] != 0) return;
  const GcibStencil s = st[i];
  int cols[5];
  double vals[5];
  const int m = merge_row(s, cols, vals);
  int nz = 0;
  for (int q = 0; q < m; ++q) nz += vals[q] != 0.;
  const int r0 = rp[s.cell], r1 = rp[s.cell + 1];
  // an IB row holds exactly its non-zero stencil entries
  if (r1 - r0 != nz) {
    counters[3] = 1;
    return;
  }
  for (int q = 0; q < m; ++q) {
    if (vals[q] == 0.) continue;
    int p = r0;
    while (p < r1 && ci[p] != cols[q]) ++p;
    if (p == r1) {
      counters[3] = 1;
      return;
    }
    base_vals[p] = vals[q];
  }
}

__global__ void k_gcib_rhs(int n, const int32_t *__restrict__ cls, int fixed,
                           double ib_ref, double *__restrict__ base_rhs) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  const int k = cls[c];
  if (k == 1) base_rhs[c] = 0. - ib_ref;
  else if (k == 2) base_rhs[c] = fixed ? -ib_ref : 0.;
}

// The mesh-static builder data, made once per mesh.
int gcib_mesh_setup(const pg_mesh *m) {
  std::lock_guard<std::mutex> lock(m->gcib_mu);
  if (m->gcib) return PG_OK;
  const HostMesh &h = m->h;
  const int64_t n = h.n_cells, nn = (int64_t)h.node_x.size();
  PG_CHECK_ARG(nn > 0 && (int64_t)h.cind.size() < INT32_MAX,
               "ghost-cell IB: mesh too large for the stencil builder");
  auto g = std::make_unique<GcibMesh>();
  std::vector<int32_t> cptr(n + 1), cind(h.cind.size());
  for (int64_t c = 0; c <= n; ++c) cptr[c] = (int32_t)h.cptr[c];
  for (size_t k = 0; k < h.cind.size(); ++k) cind[k] = (int32_t)h.cind[k];
  // node -> cells, each node's cells in increasing id (Node::cells order)
  std::vector<int32_t> nptr(nn + 1, 0), ncell(h.cind.size());
  for (size_t k = 0; k < h.cind.size(); ++k) ++nptr[cind[k] + 1];
  for (int64_t v = 0; v < nn; ++v) nptr[v + 1] += nptr[v];
  {
    std::vector<int32_t> fill(nptr.begin(), nptr.end() - 1);
    for (int64_t c = 0; c < n; ++c)
      for (int32_t k = cptr[c]; k < cptr[c + 1]; ++k)
        ncell[fill[cind[k]]++] = (int32_t)c;
  }
  // bucket grid: about four nodes per bucket
  double x0 = h.node_x[0], y0 = h.node_y[0], x1 = x0, y1 = y0;
  for (int64_t v = 0; v < nn; ++v) {
    x0 = std::min(x0, h.node_x[v]);
    y0 = std::min(y0, h.node_y[v]);
    x1 = std::max(x1, h.node_x[v]);
    y1 = std::max(y1, h.node_y[v]);
  }
  const double w = std::max(x1 - x0, 1e-300), hh = std::max(y1 - y0, 1e-300);
  const double bh = std::sqrt(w * hh / (double)nn) * 2.;
  PG_CHECK_ARG(std::isfinite(bh) && bh > 0.,
               "ghost-cell IB: degenerate node coordinates");
  const int nx = std::max(1, (int)std::min(4096., std::ceil(w / bh)));
  const int ny = std::max(1, (int)std::min(4096., std::ceil(hh / bh)));
  const double hb = std::max(w / nx, hh / ny);  // square buckets covering all
  auto bucket = [&](double v, double v0, int nb) {
    double f = std::floor((v - v0) / hb);
    f = std::min(std::max(f, 0.), (double)(nb - 1));
    return (int)f;
  };
  std::vector<int32_t> start((size_t)nx * ny + 1, 0), items(nn);
  std::vector<int32_t> bof(nn);
  for (int64_t v = 0; v < nn; ++v) {
    bof[v] = bucket(h.node_y[v], y0, ny) * nx + bucket(h.node_x[v], x0, nx);
    ++start[bof[v] + 1];
  }
  for (size_t b = 1; b < start.size(); ++b) start[b] += start[b - 1];
  {
    std::vector<int32_t> fill(start.begin(), start.end() - 1);
    for (int64_t v = 0; v < nn; ++v) items[fill[bof[v]]++] = (int32_t)v;
  }
  g->x0 = x0;
  g->y0 = y0;
  g->h = hb;
  g->nx = nx;
  g->ny = ny;
  cudaError_t ce = cudaSuccess;
  auto up = [&](auto &buf, const auto &vec) {
    if (ce == cudaSuccess) ce = buf.upload(vec);
  };
  up(g->cptr, cptr);
  up(g->cind, cind);
  up(g->nptr, nptr);
  up(g->ncell, ncell);
  up(g->bstart, start);
  up(g->bitems, items);
  up(g->node_x, h.node_x);
  up(g->node_y, h.node_y);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(stream());
  if (ce != cudaSuccess) return cuda_fail(ce, "ghost-cell IB mesh upload", __FILE__, __LINE__);
  m->gcib = std::move(g);
  return PG_OK;
}

}  // namespace

int gcib_build(const pg_mesh *m, GcibState &S, int n_circles,
               const double *circles, GcibRows &g, bool check_pattern,
               const int32_t *row_ptr, const int32_t *col_ind,
               double *base_vals, double *base_rhs, bool *changed) {
  PG_CHECK_ARG(n_circles >= 0 && (n_circles == 0 || circles),
               "ghost-cell IB: bad circles");
  PG_CHECK_ARG(S.ib_bc == PG_BC_FIXED || S.ib_bc == PG_BC_NORMAL_GRADIENT,
               "ghost-cell IB: IB boundary type must be FIXED or "
               "NORMAL_GRADIENT");
  PG_CHECK_ARG(std::isfinite(S.ib_ref), "ghost-cell IB: ib_ref not finite");
  for (int k = 0; k < n_circles; ++k)
    PG_CHECK_ARG(std::isfinite(circles[3 * k]) &&
                     std::isfinite(circles[3 * k + 1]) &&
                     std::isfinite(circles[3 * k + 2]) && circles[3 * k + 2] > 0.,
                 "ghost-cell IB: circle radius must be positive (and every "
                 "value finite)");
  PG_CHECK_ARG(!check_pattern || (row_ptr && col_ind && base_vals && base_rhs &&
                                  S.cls.p),
               "ghost-cell IB: no equation to update");
  int rc = gcib_mesh_setup(m);
  if (rc) return rc;
  const GcibMesh &gm = *m->gcib;
  const int64_t n = m->h.n_cells;
  PG_CHECK_ARG(n < INT32_MAX, "ghost-cell IB: too many cells");
  cudaStream_t st = stream();
  PG_CUDA(S.circles.upload(circles, 3 * (size_t)n_circles));
  PG_CUDA(S.new_cls.reserve(n));
  PG_CUDA(S.ib.reserve(n));
  PG_CUDA(S.counters.reserve(4));
  int32_t hc[4] = {0, 0, INT_MAX, 0};
  PG_CUDA(cudaMemcpyAsync(S.counters.p, hc, sizeof(hc), cudaMemcpyHostToDevice, st));
  const int T = 256;
  k_gcib_classify<<<(unsigned)((n + T - 1) / T), T, 0, st>>>(
      (int)n, m->d.cx.p, m->d.cy.p, n_circles, S.circles.p, gm.cptr.p,
      gm.cind.p, gm.nptr.p, gm.ncell.p, check_pattern ? S.cls.p : nullptr,
      S.new_cls.p, S.ib.p, S.counters.p);
  PG_CUDA(cudaGetLastError());
  PG_CUDA(cudaMemcpyAsync(hc, S.counters.p, sizeof(hc), cudaMemcpyDeviceToHost, st));
  PG_CUDA(cudaStreamSynchronize(st));
  const int n_ib = hc[0];
  PG_CUDA(S.st.reserve(std::max(n_ib, 1)));
  if (n_ib > 0) {
    NodeGridDev ng{gm.bstart.p, gm.bitems.p, gm.node_x.p, gm.node_y.p,
                   gm.x0, gm.y0, gm.h, gm.nx, gm.ny};
    k_gcib_stencil<<<(n_ib + T - 1) / T, T, 0, st>>>(
        n_ib, S.ib.p, S.circles.p, S.ib_bc, m->d.cx.p, m->d.cy.p, ng,
        gm.nptr.p, gm.ncell.p, S.st.p, S.counters.p);
    PG_CUDA(cudaGetLastError());
  }
  const bool same_classes = check_pattern && hc[3] == 0;
  if (same_classes && n_ib > 0) {
    k_gcib_scatter<<<(n_ib + T - 1) / T, T, 0, st>>>(n_ib, S.st.p, row_ptr,
                                                     col_ind, base_vals,
                                                     S.counters.p);
    PG_CUDA(cudaGetLastError());
  }
  PG_CUDA(cudaMemcpyAsync(hc, S.counters.p, sizeof(hc), cudaMemcpyDeviceToHost, st));
  PG_CUDA(cudaStreamSynchronize(st));
  if (hc[1] != 0) {
    const int c = hc[2];
    set_error(std::string("ghost-cell IB: ") +
              (hc[1] == 1 ? "the node nearest to the image point of IB cell " +
                                std::to_string(c) + " does not have four cells"
                          : "singular IB stencil at cell " + std::to_string(c)));
    return PG_BAD_ARG;
  }
  const bool ch = !check_pattern || hc[3] != 0;
  if (!ch) {
    k_gcib_rhs<<<(unsigned)((n + T - 1) / T), T, 0, st>>>(
        (int)n, S.new_cls.p, S.ib_bc == PG_BC_FIXED, S.ib_ref, base_rhs);
    PG_CUDA(cudaGetLastError());
  } else {
    // the rows of the new pattern, as the host pattern builder takes them
    std::vector<GcibStencil> recs(n_ib);
    g.cls.resize(n);
    PG_CUDA(cudaMemcpyAsync(g.cls.data(), S.new_cls.p, n * sizeof(int32_t),
                            cudaMemcpyDeviceToHost, st));
    if (n_ib > 0)
      PG_CUDA(cudaMemcpyAsync(recs.data(), S.st.p, n_ib * sizeof(GcibStencil),
                              cudaMemcpyDeviceToHost, st));
    PG_CUDA(cudaStreamSynchronize(st));
    g.rows.assign(n, {});
    g.rhs.assign(n, 0.);
    auto add = [&](int64_t row, int32_t col, double v) {
      for (auto &e : g.rows[row])
        if (e.first == col) {
          e.second += v;
          return;
        }
      g.rows[row].push_back({col, v});
    };
    for (const GcibStencil &s : recs) {
      for (int j = 0; j < 4; ++j) add(s.cell, s.st[j], s.co[j]);
      if (s.has_self) add(s.cell, s.cell, s.self);
      g.rhs[s.cell] += -S.ib_ref;
    }
    for (int64_t c = 0; c < n; ++c) {
      if (g.cls[c] != 2) continue;
      add(c, (int32_t)c, 1.);
      g.rhs[c] = S.ib_bc == PG_BC_FIXED ? -S.ib_ref : 0.;
    }
    // CrsEquation::operator+ keeps only non-zero entries
    for (auto &row : g.rows) {
      std::vector<std::pair<int32_t, double>> kept;
      for (auto &e : row)
        if (e.second != 0.) kept.push_back(e);
      row.swap(kept);
    }
  }
  std::swap(S.cls.p, S.new_cls.p);
  std::swap(S.cls.n, S.new_cls.n);
  S.n_ib = n_ib;
  S.n_circles = n_circles;
  if (changed) *changed = ch;
  return PG_OK;
}

}  // namespace pg
