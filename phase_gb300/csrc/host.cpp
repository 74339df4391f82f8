// Host-side set-up of libphase_gb300: mesh construction, the CrsEquation
// sparsity pattern with its face-coloured scatter schedule, and the sparsity
// analysis (Schwarz partition + level schedule) of solver matrices.
// All of it runs once per mesh / per pattern, never per solve.
// Built with -ffp-contract=off so geometry rounds as the reference's does.
#include <algorithm>
#include <cstdlib>
#include <cmath>
#include <cstring>
#include <map>
#include <numeric>
#include <string>
#include <tuple>

#include "internal.h"

namespace pg {

// ------------------------------------------------------------------ mesh
// FiniteVolumeGrid2D::init(nodes, cptr, cind) (FiniteVolumeGrid2D.cpp:20-35)
// and createCell (:84-114).  Faces are de-duplicated on their unordered node
// pair with a per-node adjacency chain (no ordered map): the first cell that
// meets a face creates it with (lNode, rNode) in that cell's orientation and
// becomes its lCell; the second cell makes it interior as rCell.
int build_host_mesh(const double *nodes_xy, int64_t n_nodes,
                    const int64_t *cptr, const int64_t *cind, int64_t n_cells,
                    HostMesh &m) {
  PG_CHECK_ARG(nodes_xy && cptr && cind, "pg_mesh_create: NULL array");
  PG_CHECK_ARG(n_nodes > 0 && n_cells > 0, "pg_mesh_create: empty mesh");
  PG_CHECK_ARG(n_cells < (int64_t)1 << 30, "pg_mesh_create: too many cells");
  PG_CHECK_ARG(cptr[0] == 0, "pg_mesh_create: cptr[0] must be 0");
  for (int64_t c = 0; c < n_cells; ++c)
    PG_CHECK_ARG(cptr[c + 1] - cptr[c] >= 3,
                 "pg_mesh_create: a cell needs at least 3 nodes");
  const int64_t n_ent = cptr[n_cells];
  for (int64_t k = 0; k < n_ent; ++k)
    PG_CHECK_ARG(cind[k] >= 0 && cind[k] < n_nodes,
                 "pg_mesh_create: node index out of range");

  m.n_cells = n_cells;
  m.node_x.resize(n_nodes);
  m.node_y.resize(n_nodes);
  for (int64_t i = 0; i < n_nodes; ++i) {
    m.node_x[i] = nodes_xy[2 * i];
    m.node_y[i] = nodes_xy[2 * i + 1];
  }
  m.cptr.assign(cptr, cptr + n_cells + 1);
  m.cind.assign(cind, cind + cptr[n_cells]);
  m.cx.resize(n_cells);
  m.cy.resize(n_cells);
  m.vol.resize(n_cells);

  std::vector<int32_t> head(n_nodes, -1), next, other, fid;
  next.reserve(n_ent);
  other.reserve(n_ent);
  fid.reserve(n_ent);
  m.fl.reserve(n_ent / 2 + 16);

  for (int64_t c = 0; c < n_cells; ++c) {
    const int64_t b = cptr[c], k = cptr[c + 1] - b;
    // Cell::Cell (Cell.cpp:8-29): polygon area and centroid from the
    // shoelace sums; orientation is corrected so the area is positive.
    double a2 = 0., sx = 0., sy = 0.;
    for (int64_t i = 0; i < k; ++i) {
      const int64_t p = cind[b + i], q = cind[b + (i + 1) % k];
      const double px = nodes_xy[2 * p], py = nodes_xy[2 * p + 1];
      const double qx = nodes_xy[2 * q], qy = nodes_xy[2 * q + 1];
      const double cr = px * qy - qx * py;
      a2 += cr;
      sx += (px + qx) * cr;
      sy += (py + qy) * cr;
    }
    PG_CHECK_ARG(a2 != 0., "pg_mesh_create: degenerate (zero-area) cell");
    m.vol[c] = std::fabs(a2) / 2.;
    m.cx[c] = sx / (3. * a2);
    m.cy[c] = sy / (3. * a2);

    for (int64_t i = 0; i < k; ++i) {
      const int32_t n1 = (int32_t)cind[b + i];
      const int32_t n2 = (int32_t)cind[b + (i + 1) % k];
      const int32_t lo = std::min(n1, n2), hi = std::max(n1, n2);
      int32_t found = -1;
      for (int32_t e = head[lo]; e >= 0; e = next[e])
        if (other[e] == hi) {
          found = fid[e];
          break;
        }
      if (found < 0) {
        const int32_t f = (int32_t)m.fl.size();
        next.push_back(head[lo]);
        other.push_back(hi);
        fid.push_back(f);
        head[lo] = (int32_t)next.size() - 1;
        // Face::Face (Face.cpp:9-18): centroid 0.5*(l + r), tangent r - l,
        // normal = tangent.normalVec() = (t.y, -t.x) (Vector2D.h:26)
        const double lx = nodes_xy[2 * n1], ly = nodes_xy[2 * n1 + 1];
        const double rx = nodes_xy[2 * n2], ry = nodes_xy[2 * n2 + 1];
        m.fcx.push_back(0.5 * (lx + rx));
        m.fcy.push_back(0.5 * (ly + ry));
        m.fnx.push_back(ry - ly);
        m.fny.push_back(-(rx - lx));
        m.fl.push_back((int32_t)c);
        m.fr.push_back(-1);
      } else {
        // Face::addCell (Face.cpp:66-81): at most two cells per face
        PG_CHECK_ARG(m.fr[found] < 0,
                     "pg_mesh_create: a face is shared by more than two cells");
        m.fr[found] = (int32_t)c;
      }
    }
  }
  m.n_faces = (int64_t)m.fl.size();

  // FiniteVolumeGrid2D::init() (:405-419): walk faces in id order; boundary
  // faces give their lCell a boundary link, interior faces give both cells an
  // interior link.  Per cell the interior links precede the boundary links.
  std::vector<int32_t> ni(n_cells, 0), nb(n_cells, 0);
  for (int64_t f = 0; f < m.n_faces; ++f) {
    if (m.fr[f] < 0) {
      ++nb[m.fl[f]];
      ++m.n_boundary;
    } else {
      ++ni[m.fl[f]];
      ++ni[m.fr[f]];
      ++m.n_interior;
    }
  }
  m.link_ptr.assign(n_cells + 1, 0);
  for (int64_t c = 0; c < n_cells; ++c)
    m.link_ptr[c + 1] = m.link_ptr[c] + ni[c] + nb[c];
  m.link_face.assign(m.link_ptr[n_cells], -1);
  m.link_cell.assign(m.link_ptr[n_cells], -1);
  std::vector<int64_t> pi(n_cells), pb(n_cells);
  for (int64_t c = 0; c < n_cells; ++c) {
    pi[c] = m.link_ptr[c];
    pb[c] = m.link_ptr[c] + ni[c];
  }
  for (int32_t f = 0; f < (int32_t)m.n_faces; ++f) {
    const int32_t l = m.fl[f], r = m.fr[f];
    if (r < 0) {
      m.link_face[pb[l]++] = f;
    } else {
      m.link_face[pi[l]] = f;
      m.link_cell[pi[l]++] = r;
      m.link_face[pi[r]] = f;
      m.link_cell[pi[r]++] = l;
    }
  }
  m.n_interior_links = std::move(ni);
  return PG_OK;
}

// ---------------------------------------------------------------- pattern
// The pattern CrsEquation holds after fv::laplacian: each row starts with 5
// placeholder slots (CrsEquation.cpp:9-14) that addCoeff fills in order of
// first appearance of a column, appending past the fifth (:113-131).  The
// scalar-gamma overload adds (cell, nb) before (cell, cell) for every
// interior link (Laplacian.h:55-58); the face-gamma overload adds the
// diagonal first (:139-142); FIXED boundary links add the diagonal
// (:66-69, :150-153).  Placeholders that stay empty are dropped.
int build_pattern(const HostMesh &m, int gamma_kind, const int32_t *bc_type,
                  EqnPattern &p, bool diag_first, const GcibRows *extra) {
  const int64_t n = m.n_cells;
  p.n = n;
  p.row_ptr.assign(n + 1, 0);
  p.col_ind.clear();
  p.col_ind.reserve(n * 5);
  p.diag.assign(n, -1);
  const int64_t nf = m.n_faces;
  std::vector<int32_t> f_slot_l(nf, -1), f_slot_r(nf, -1), f_diag_l(nf, -1),
      f_diag_r(nf, -1);

  std::vector<int32_t> row;
  auto add = [&](int32_t col) -> int32_t {
    for (size_t k = 0; k < row.size(); ++k)
      if (row[k] == col) return (int32_t)k;
    row.push_back(col);
    return (int32_t)row.size() - 1;
  };
  for (int64_t c = 0; c < n; ++c) {
    row.clear();
    if (diag_first) add((int32_t)c);  // fv::ddt's diagonal comes first
    const bool fluid = !extra || extra->cls[c] == 0;
    const int64_t b = fluid ? m.link_ptr[c] : 0, e = fluid ? m.link_ptr[c + 1] : 0;
    const int64_t base = (int64_t)p.col_ind.size();
    if (extra)  // CrsEquation::operator+ appends the IB row's entries
      for (const auto &en : extra->rows[c]) add(en.first);
    for (int64_t k = b; k < e; ++k) {
      const int32_t f = m.link_face[k], nbc = m.link_cell[k];
      if (nbc >= 0) {
        int32_t so, sd;
        if (gamma_kind == PG_GAMMA_FACE) {
          sd = add((int32_t)c);
          so = add(nbc);
        } else {
          so = add(nbc);
          sd = add((int32_t)c);
        }
        const bool is_l = m.fl[f] == (int32_t)c;
        (is_l ? f_slot_l : f_slot_r)[f] = (int32_t)(base + so);
        (is_l ? f_diag_l : f_diag_r)[f] = (int32_t)(base + sd);
      } else if (bc_type[f] == PG_BC_FIXED) {
        f_diag_l[f] = (int32_t)(base + add((int32_t)c));
      }
    }
    for (size_t k = 0; k < row.size(); ++k) {
      if (row[k] == (int32_t)c) p.diag[c] = (int32_t)(base + k);
      p.col_ind.push_back(row[k]);
    }
    PG_CHECK_ARG(p.col_ind.size() < ((size_t)1 << 31),
                 "pg_eqn_create: too many matrix entries");
    p.row_ptr[c + 1] = (int32_t)p.col_ind.size();
  }
  p.nnz = (int64_t)p.col_ind.size();

  // Greedy face colouring in face-id order: a face takes the lowest colour
  // that no other face of its cells has; interior faces use colours
  // [0, n_interior_colors), boundary faces the colours after them.  Faces of
  // one colour share no cell, so one launch per colour scatters into the
  // diagonal and the rhs of both cells without atomics.
  std::vector<uint64_t> used(n, 0);
  std::vector<int32_t> color(nf, -1);
  int max_c = -1;
  for (int64_t f = 0; f < nf; ++f) {
    if (m.fr[f] < 0) continue;
    uint64_t u = used[m.fl[f]] | used[m.fr[f]];
    PG_CHECK_ARG(~u != 0, "pg_eqn_create: more than 64 face colours");
    int cidx = __builtin_ctzll(~u);
    color[f] = cidx;
    used[m.fl[f]] |= 1ull << cidx;
    used[m.fr[f]] |= 1ull << cidx;
    max_c = std::max(max_c, cidx);
  }
  p.n_interior_colors = max_c + 1;
  std::fill(used.begin(), used.end(), 0);
  int max_b = -1;
  for (int64_t f = 0; f < nf; ++f) {
    if (m.fr[f] >= 0) continue;
    uint64_t u = used[m.fl[f]];
    PG_CHECK_ARG(~u != 0, "pg_eqn_create: more than 64 boundary face colours");
    int cidx = __builtin_ctzll(~u);
    used[m.fl[f]] |= 1ull << cidx;
    color[f] = p.n_interior_colors + cidx;
    max_b = std::max(max_b, cidx);
  }
  const int n_colors = p.n_interior_colors + max_b + 1;
  p.color_ptr.assign(n_colors + 1, 0);
  for (int64_t f = 0; f < nf; ++f) ++p.color_ptr[color[f] + 1];
  for (int c = 0; c < n_colors; ++c) p.color_ptr[c + 1] += p.color_ptr[c];
  std::vector<int32_t> fill(p.color_ptr.begin(), p.color_ptr.end() - 1);
  p.cface.assign(nf, -1);
  for (int32_t f = 0; f < (int32_t)nf; ++f) p.cface[fill[color[f]]++] = f;
  p.slot_lr.resize(nf);
  p.slot_rl.resize(nf);
  p.diag_l.resize(nf);
  p.diag_r.resize(nf);
  for (int64_t k = 0; k < nf; ++k) {
    const int32_t f = p.cface[k];
    p.slot_lr[k] = f_slot_l[f];
    p.slot_rl[k] = f_slot_r[f];
    p.diag_l[k] = f_diag_l[f];
    p.diag_r[k] = f_diag_r[f];
  }
  return PG_OK;
}

// --------------------------------------------------------------- analysis
namespace {

// Recursive graph bisection on the symmetrised pattern.  Each range of
// vertices is reordered by breadth-first distance from a pseudo-peripheral
// vertex (two sweeps) and cut so both halves hold whole multiples of the
// target subdomain size; cuts recurse until a range fits one subdomain.
// (With row coordinates, analyse() cuts by coordinate instead.)
// Emission order is left-to-right, so consecutive subdomains are neighbours.
struct Bisector {
  int64_t n;
  const std::vector<int64_t> &ap;
  const std::vector<int32_t> &aj;
  std::vector<int32_t> in_range, seen;
  int32_t range_stamp = 0, seen_stamp = 0;
  std::vector<int32_t> queue;

  Bisector(int64_t n_, const std::vector<int64_t> &ap_,
           const std::vector<int32_t> &aj_)
      : n(n_), ap(ap_), aj(aj_), in_range(n_, 0), seen(n_, 0) {
    queue.reserve(n_);
  }

  // BFS over the vertices stamped in_range, starting at s and restarting at
  // unvisited vertices of `verts` so disconnected ranges are covered.
  // Returns the last vertex dequeued; the visit order is left in `queue`.
  int32_t bfs(int32_t s, const int32_t *verts, int64_t cnt) {
    ++seen_stamp;
    queue.clear();
    int64_t head = 0, scan = 0;
    int32_t last = s;
    auto push = [&](int32_t v) {
      seen[v] = seen_stamp;
      queue.push_back(v);
    };
    push(s);
    while ((int64_t)queue.size() < cnt) {
      while (head < (int64_t)queue.size()) {
        int32_t v = queue[head++];
        last = v;
        for (int64_t k = ap[v]; k < ap[v + 1]; ++k) {
          int32_t w = aj[k];
          if (in_range[w] == range_stamp && seen[w] != seen_stamp) push(w);
        }
      }
      while ((int64_t)queue.size() < cnt && seen[verts[scan]] == seen_stamp)
        ++scan;
      if ((int64_t)queue.size() < cnt) push(verts[scan]);
    }
    while (head < (int64_t)queue.size()) last = queue[head++];
    return last;
  }
};

}  // namespace

// ILU(k) pattern of one subdomain by levels of fill (Saad, Iterative
// Methods for Sparse Linear Systems, 2nd ed., sec. 10.3.3; Ifpack2 RILUK's
// "fact: iluk level-of-fill"): rows in increasing index, the entries of A
// inside the subdomain at level 0, and a fill entry (i, j) at level
// lev(i,k) + lev(k,j) + 1 for every k < i in row i's pattern and j > k in
// row k's; entries above level p are dropped.  out[r] receives row r's
// columns (original ids, ascending, diagonal included) for every r in rows.
static void iluk_pattern(const std::vector<int32_t> &rows, int s,
                         const std::vector<int64_t> &cp,
                         const std::vector<int32_t> &cc,
                         const std::vector<int32_t> &part, int p,
                         std::vector<std::vector<int32_t>> &out) {
  const size_t nr = rows.size();
  auto local = [&](int32_t r) {
    return (int32_t)(std::lower_bound(rows.begin(), rows.end(), r) - rows.begin());
  };
  // per local row: its U part (local col > row) with levels, for later rows
  std::vector<std::vector<std::pair<int32_t, int32_t>>> upart(nr);
  std::map<int32_t, int32_t> lev;  // local col -> level
  for (size_t i = 0; i < nr; ++i) {
    lev.clear();
    const int32_t r = rows[i];
    lev[(int32_t)i] = 0;
    for (int64_t k = cp[r]; k < cp[r + 1]; ++k)
      if (part[cc[k]] == s) lev[local(cc[k])] = 0;
    for (auto it = lev.begin(); it != lev.end() && it->first < (int32_t)i; ++it) {
      const int32_t k = it->first, lik = it->second;
      if (lik > p) continue;
      for (const auto &e : upart[k]) {
        const int32_t lnew = lik + e.second + 1;
        if (lnew > p) continue;
        auto f = lev.find(e.first);
        if (f == lev.end()) lev.emplace(e.first, lnew);
        else if (lnew < f->second) f->second = lnew;
      }
    }
    std::vector<int32_t> &cols = out[r];
    cols.clear();
    for (const auto &e : lev) {
      if (e.second > p) continue;
      cols.push_back(rows[e.first]);
      if (e.first > (int32_t)i) upart[i].push_back(e);
    }
  }
}

// Grid coordinates of a subdomain that is a rectangular block of a
// structured grid with a 5-point pattern: every in-subdomain neighbour of a
// row is one level before or after it and is the row's neighbour along one
// grid axis, and the block is full (W x H rows).  Coordinates are built level
// by level: the level-0 row is the corner (0, 0); of the two level-1 rows the
// one with the smaller index is (1, 0); a row with two earlier neighbours
// (i-1, j) and (i, j-1) is (i, j); a row with one earlier neighbour extends
// the edge that neighbour lies on.  Lines run along the shorter side
// (gline = the line, gpos = the position along it).  Returns the number of
// lines, or 0 when the subdomain is not such a block.
static int grid_block(const std::vector<int32_t> &rows, int s,
               const std::vector<int32_t> &level,
               const std::vector<int64_t> &ap, const std::vector<int32_t> &aj,
               const std::vector<int32_t> &part, std::vector<int32_t> &gline,
               std::vector<int32_t> &gpos) {
  const int64_t nr = (int64_t)rows.size();
  if (nr < 2 || nr > 65535) return 0;
  int32_t nlev = 0;
  for (int32_t r : rows) nlev = std::max(nlev, level[r] + 1);
  if (nlev < 2) return 0;
  std::vector<std::vector<int32_t>> by_level(nlev);
  for (int32_t r : rows) by_level[level[r]].push_back(r);  // index order
  if (by_level[0].size() != 1 || by_level[1].empty() || by_level[1].size() > 2)
    return 0;
  std::vector<int32_t> ci(nr), cj(nr);
  auto slot = [&](int32_t r) {  // position of r in rows
    return std::lower_bound(rows.begin(), rows.end(), r) - rows.begin();
  };
  ci[slot(by_level[0][0])] = 0;
  cj[slot(by_level[0][0])] = 0;
  int32_t W = 1, H = 1;
  for (int32_t l = 1; l < nlev; ++l) {
    for (size_t q = 0; q < by_level[l].size(); ++q) {
      const int32_t r = by_level[l][q];
      int32_t lnb[2], nlnb = 0;
      for (int64_t k = ap[r]; k < ap[r + 1]; ++k) {
        const int32_t c = aj[k];
        if (part[c] != s) continue;
        if (level[c] == l - 1) {
          if (nlnb == 2) return 0;
          lnb[nlnb++] = c;
        } else if (level[c] != l + 1) {
          return 0;
        }
      }
      int32_t i, j;
      if (nlnb == 2) {
        const int64_t p = slot(lnb[0]), qq = slot(lnb[1]);
        i = std::max(ci[p], ci[qq]);
        j = std::max(cj[p], cj[qq]);
        const bool ok = (ci[p] == i - 1 && cj[p] == j && ci[qq] == i && cj[qq] == j - 1) ||
                        (ci[qq] == i - 1 && cj[qq] == j && ci[p] == i && cj[p] == j - 1);
        if (!ok) return 0;
      } else if (nlnb == 1) {
        const int64_t p = slot(lnb[0]);
        if (l == 1) {
          i = q == 0 ? 1 : 0;
          j = q == 0 ? 0 : 1;
        } else if (cj[p] == 0 && ci[p] > 0) {
          i = ci[p] + 1;
          j = 0;
        } else if (ci[p] == 0 && cj[p] > 0) {
          i = 0;
          j = cj[p] + 1;
        } else {
          return 0;
        }
      } else {
        return 0;
      }
      const int64_t sr = slot(r);
      ci[sr] = i;
      cj[sr] = j;
      W = std::max(W, i + 1);
      H = std::max(H, j + 1);
    }
  }
  if ((int64_t)W * H != nr) return 0;
  std::vector<int32_t> grid((size_t)W * H, -1);
  for (int64_t k = 0; k < nr; ++k) {
    int32_t &g = grid[(size_t)cj[k] * W + ci[k]];
    if (g >= 0) return 0;
    g = (int32_t)k;
  }
  // every in-subdomain neighbour is a grid neighbour
  for (int64_t k = 0; k < nr; ++k) {
    const int32_t r = rows[k];
    for (int64_t e = ap[r]; e < ap[r + 1]; ++e) {
      const int32_t c = aj[e];
      if (part[c] != s) continue;
      const int64_t p = slot(c);
      if (std::abs(ci[p] - ci[k]) + std::abs(cj[p] - cj[k]) != 1) return 0;
    }
  }
  const bool swap = W > H;
  for (int64_t k = 0; k < nr; ++k) {
    gline[rows[k]] = swap ? cj[k] : ci[k];
    gpos[rows[k]] = swap ? ci[k] : cj[k];
  }
  return swap ? H : W;
}

int analyse(int64_t n, const int32_t *row_ptr, const int32_t *col_ind,
            int subdomain_rows, Analysis &a,
            const std::vector<int64_t> *sys_rows, const double *cx,
            const double *cy, int fill) {
  PG_CHECK_ARG(n > 0 && row_ptr && col_ind, "analyse: empty matrix");
  PG_CHECK_ARG(row_ptr[0] == 0, "row_ptr[0] must be 0");
  for (int64_t i = 0; i < n; ++i)
    PG_CHECK_ARG(row_ptr[i + 1] >= row_ptr[i], "row_ptr must be non-decreasing");
  const int64_t n_src = row_ptr[n];
  for (int64_t k = 0; k < n_src; ++k)
    PG_CHECK_ARG(col_ind[k] < n, "column index out of range");

  a = Analysis();
  a.n = n;
  a.n_src = n_src;

  // 1. compact rows: drop placeholders, merge repeated columns
  std::vector<int64_t> cp(n + 1, 0);
  std::vector<int32_t> cc, cs;  // column, source index
  cc.reserve(n_src);
  cs.reserve(n_src);
  {
    std::vector<int32_t> mark(n, -1);
    for (int64_t i = 0; i < n; ++i) {
      const int64_t start = (int64_t)cc.size();
      for (int64_t k = row_ptr[i]; k < row_ptr[i + 1]; ++k) {
        const int32_t c = col_ind[k];
        if (c < 0) continue;
        if (mark[c] >= start) {  // repeated column: summed later
          a.dup_src.push_back((int32_t)k);
          a.dup_dst.push_back(mark[c]);  // compact index, remapped below
          continue;
        }
        mark[c] = (int32_t)cc.size();
        cc.push_back(c);
        cs.push_back((int32_t)k);
      }
      cp[i + 1] = (int64_t)cc.size();
    }
  }
  a.nnz = (int64_t)cc.size();

  // 2. symmetrised adjacency without the diagonal
  std::vector<int64_t> ap(n + 1, 0);
  std::vector<int32_t> aj;
  {
    std::vector<int64_t> deg(n, 0);
    for (int64_t i = 0; i < n; ++i)
      for (int64_t k = cp[i]; k < cp[i + 1]; ++k)
        if (cc[k] != i) {
          ++deg[i];
          ++deg[cc[k]];
        }
    for (int64_t i = 0; i < n; ++i) ap[i + 1] = ap[i] + deg[i];
    aj.resize(ap[n]);
    std::vector<int64_t> pos(ap.begin(), ap.end() - 1);
    for (int64_t i = 0; i < n; ++i)
      for (int64_t k = cp[i]; k < cp[i + 1]; ++k)
        if (cc[k] != i) {
          aj[pos[i]++] = cc[k];
          aj[pos[cc[k]]++] = (int32_t)i;
        }
    // sort + unique each list
    std::vector<int64_t> np(n + 1, 0);
    int64_t w = 0;
    for (int64_t i = 0; i < n; ++i) {
      std::sort(aj.begin() + ap[i], aj.begin() + ap[i + 1]);
      int64_t e = std::unique(aj.begin() + ap[i], aj.begin() + ap[i + 1]) -
                  aj.begin();
      for (int64_t k = ap[i]; k < e; ++k) aj[w++] = aj[k];
      np[i + 1] = w;
    }
    aj.resize(w);
    ap.swap(np);
  }

  // 3. partition
  int64_t target = subdomain_rows;
  if (target == 0) target = 1024;
  std::vector<int32_t> order(n);
  std::iota(order.begin(), order.end(), 0);
  std::vector<std::pair<int64_t, int64_t>> parts;  // ranges of `order`
  if (!sys_rows && (target < 0 || n <= target)) {
    parts.push_back({0, n});
    a.global_ilu = (target < 0) || n <= target;
  } else {
    if (target < 0) target = INT32_MAX;
    Bisector bs(n, ap, aj);
    // ranges to cut; the flag marks a range whose cut was moved to a grid
    // line, which may then hold up to a quarter more than the target
    std::vector<std::tuple<int64_t, int64_t, bool>> stack{{0, n, false}};
    const bool rcb = cx && cy;
    if (sys_rows) {  // one root range per system, popped in system order
      PG_CHECK_ARG(sys_rows->size() >= 2 && sys_rows->front() == 0 &&
                       sys_rows->back() == n,
                   "analyse: bad system row offsets");
      stack.clear();
      for (size_t k = sys_rows->size() - 1; k-- > 0;)
        if ((*sys_rows)[k + 1] > (*sys_rows)[k])
          stack.push_back({(*sys_rows)[k], (*sys_rows)[k + 1], false});
    }
    while (!stack.empty()) {
      auto [lo, hi, snapped] = stack.back();
      stack.pop_back();
      const int64_t cnt = hi - lo;
      if (cnt <= target || (snapped && cnt <= target + target / 4)) {
        parts.push_back({lo, hi});
        continue;
      }
      const int64_t k_parts = (cnt + target - 1) / target;
      int64_t left = cnt * (k_parts / 2) / k_parts;
      if (rcb) {
        // coordinate bisection across the longer extent of the range's
        // cell centres (ties broken by row index)
        double x0 = cx[order[lo]], x1 = x0, y0 = cy[order[lo]], y1 = y0;
        for (int64_t k = lo; k < hi; ++k) {
          const int32_t r = order[k];
          x0 = std::min(x0, cx[r]), x1 = std::max(x1, cx[r]);
          y0 = std::min(y0, cy[r]), y1 = std::max(y1, cy[r]);
        }
        const double *c = x1 - x0 >= y1 - y0 ? cx : cy;
        auto by_c = [c](int32_t p, int32_t q) {
          return c[p] < c[q] || (c[p] == c[q] && p < q);
        };
        std::nth_element(order.begin() + lo, order.begin() + lo + left,
                         order.begin() + hi, by_c);
        // On a structured grid the cells of one grid line share their
        // coordinate up to rounding: move the cut to the nearer boundary of
        // the cut cell's line, so blocks stay whole rectangles (the line
        // form of the sweep needs them).  Unstructured centres are distinct
        // beyond the tolerance, and their cut does not move.
        const double tol = 1e-9 * std::max(x1 - x0, y1 - y0);
        const double cv = c[order[lo + left]];
        int64_t below = 0, upto = 0;
        for (int64_t k = lo; k < hi; ++k) {
          const double ck = c[order[k]];
          below += ck < cv - tol;
          upto += ck <= cv + tol;
        }
        int64_t cut = left;
        if (below != left) {
          const bool lo_ok = below > 0, hi_ok = upto < cnt;
          if (lo_ok && (!hi_ok || left - below <= upto - left)) cut = below;
          else if (hi_ok) cut = upto;
        }
        if (cut != left) {
          if (cut == below)
            std::partition(order.begin() + lo, order.begin() + hi,
                           [&](int32_t r) { return c[r] < cv - tol; });
          else
            std::partition(order.begin() + lo, order.begin() + hi,
                           [&](int32_t r) { return c[r] <= cv + tol; });
        }
        snapped = snapped || cut != left;
        left = cut;
      } else {
        ++bs.range_stamp;
        for (int64_t k = lo; k < hi; ++k) bs.in_range[order[k]] = bs.range_stamp;
        int32_t start = *std::min_element(order.begin() + lo, order.begin() + hi);
        int32_t far = bs.bfs(start, order.data() + lo, cnt);
        bs.bfs(far, order.data() + lo, cnt);
        std::copy(bs.queue.begin(), bs.queue.end(), order.begin() + lo);
      }
      stack.push_back({lo + left, hi, snapped});
      stack.push_back({lo, lo + left, snapped});
    }
  }
  a.n_sub = (int)parts.size();
  a.part.assign(n, 0);
  for (int s = 0; s < a.n_sub; ++s)
    for (int64_t k = parts[s].first; k < parts[s].second; ++k)
      a.part[order[k]] = s;

  // 4. levels inside each subdomain (rows visited in increasing original
  //    index; a row's level is one more than its deepest earlier neighbour
  //    in the same subdomain) and the level-ordered permutation.  A
  //    subdomain that is a rectangular block of a structured grid gets grid
  //    coordinates (line, position on the line) and each of its levels is
  //    ordered by line, for the line form of the sweep (kernels.cuh
  //    LineMeta); rows of one level are independent, so the order inside a
  //    level leaves the ILU(0) unchanged.
  std::vector<int32_t> level(n, 0);
  std::vector<int32_t> gline, gpos;  // grid coordinates of line-form rows
  std::vector<int32_t> sub_lines(a.n_sub, 0);  // lines per block, 0 = none
  // ILU(k): each row's filled pattern (original column ids)
  std::vector<std::vector<int32_t>> fill_cols(fill > 0 ? n : 0),
      fill_dep(fill > 0 ? n : 0);
  const bool want_line = !sys_rows && [] {
    const char *e = std::getenv("PG_LINE");
    return !(e && e[0] == '0');
  }();
  if (want_line) {
    gline.assign(n, -1);
    gpos.assign(n, -1);
  }
  a.perm.resize(n);
  a.sub_ptr.assign(a.n_sub + 1, 0);
  a.sub_lvl.assign(a.n_sub + 1, 0);
  a.lvl_ptr.assign(1, 0);
  int64_t out = 0;
  for (int s = 0; s < a.n_sub; ++s) {
    std::vector<int32_t> rows(order.begin() + parts[s].first,
                              order.begin() + parts[s].second);
    std::sort(rows.begin(), rows.end());
    int32_t nl = 0;
    if (fill > 0) {
      iluk_pattern(rows, s, cp, cc, a.part, fill, fill_cols);
      // the filled pattern in both directions (it need not be symmetric):
      // a row comes after every earlier row it is coupled to, so the level
      // order keeps the original order of every coupled pair
      for (int32_t r : rows) fill_dep[r].clear();
      for (int32_t r : rows)
        for (int32_t c : fill_cols[r])
          if (c > r) fill_dep[c].push_back(r);
    }
    for (int32_t i : rows) {
      int32_t lv = 0;
      if (fill > 0) {  // the filled pattern decides the schedule
        for (int32_t j : fill_cols[i])
          if (j < i) lv = std::max(lv, level[j] + 1);
        for (int32_t j : fill_dep[i]) lv = std::max(lv, level[j] + 1);
      } else {
        for (int64_t k = ap[i]; k < ap[i + 1]; ++k) {
          const int32_t j = aj[k];
          if (j < i && a.part[j] == s) lv = std::max(lv, level[j] + 1);
        }
      }
      level[i] = lv;
      nl = std::max(nl, lv + 1);
    }
    if (want_line && fill == 0)
      sub_lines[s] = grid_block(rows, s, level, ap, aj, a.part, gline, gpos);
    if (sub_lines[s] > 0)
      std::stable_sort(rows.begin(), rows.end(), [&](int32_t x, int32_t y) {
        return level[x] < level[y] ||
               (level[x] == level[y] && gline[x] < gline[y]);
      });
    else
      std::stable_sort(rows.begin(), rows.end(), [&](int32_t x, int32_t y) {
        return level[x] < level[y];
      });
    a.sub_ptr[s] = (int32_t)out;
    for (size_t k = 0; k < rows.size(); ++k) {
      if (k == 0 || level[rows[k]] != level[rows[k - 1]])
        if (k > 0) a.lvl_ptr.push_back((int32_t)(out + k));
      a.perm[out + k] = rows[k];
    }
    out += (int64_t)rows.size();
    a.lvl_ptr.push_back((int32_t)out);
    a.sub_lvl[s + 1] = (int32_t)a.lvl_ptr.size() - 1;
    a.max_sub_rows = std::max(a.max_sub_rows, (int)rows.size());
    a.max_levels = std::max(a.max_levels, (int)nl);
  }
  a.sub_ptr[a.n_sub] = (int32_t)n;
  a.iperm.resize(n);
  for (int64_t k = 0; k < n; ++k) a.iperm[a.perm[k]] = (int32_t)k;

  // 5. permuted CSR, columns sorted
  a.prp.assign(n + 1, 0);
  a.pci.resize(a.nnz);
  a.psrc.resize(a.nnz);
  std::vector<int32_t> cmap(a.nnz);  // compact index -> permuted index
  {
    std::vector<std::pair<int32_t, int32_t>> tmp;
    int64_t w = 0;
    for (int64_t i = 0; i < n; ++i) {
      const int32_t r = a.perm[i];
      tmp.clear();
      for (int64_t k = cp[r]; k < cp[r + 1]; ++k)
        tmp.push_back({a.iperm[cc[k]], (int32_t)k});
      std::sort(tmp.begin(), tmp.end());
      for (auto &t : tmp) {
        a.pci[w] = t.first;
        a.psrc[w] = cs[t.second];
        cmap[t.second] = (int32_t)w;
        ++w;
      }
      a.prp[i + 1] = (int32_t)w;
    }
  }
  for (auto &d : a.dup_dst) d = cmap[d];

  // 5a. sliced ELLPACK copy of the permuted pattern (slices of 32 rows,
  //     each as wide as its longest row, stored column-major: entry k of
  //     row r at sell_ptr[r / 32] + 32 k + r % 32), read by the FP64
  //     SpMVs so a warp's loads of one entry slot are contiguous; padding
  //     has column r and no source (value 0)
  {
    const int64_t ns = (n + 31) / 32;
    a.sell_ptr.assign(ns + 1, 0);
    for (int64_t sl = 0; sl < ns; ++sl) {
      int32_t w = 0;
      for (int64_t r = 32 * sl; r < std::min<int64_t>(n, 32 * sl + 32); ++r)
        w = std::max(w, a.prp[r + 1] - a.prp[r]);
      a.sell_ptr[sl + 1] = a.sell_ptr[sl] + 32 * w;
    }
    a.sell_col.assign(a.sell_ptr[ns], 0);
    a.sell_src.assign(a.sell_ptr[ns], -1);
    for (int64_t sl = 0; sl < ns; ++sl) {
      const int32_t w = (a.sell_ptr[sl + 1] - a.sell_ptr[sl]) / 32;
      for (int64_t r = 32 * sl; r < 32 * sl + 32; ++r) {
        const int32_t len = r < n ? a.prp[r + 1] - a.prp[r] : 0;
        for (int32_t k = 0; k < w; ++k) {
          const int64_t e = a.sell_ptr[sl] + 32 * (int64_t)k + (r - 32 * sl);
          a.sell_col[e] = k < len ? a.pci[a.prp[r] + k] : (int32_t)std::min<int64_t>(r, n - 1);
          a.sell_src[e] = k < len ? a.prp[r] + k : -1;
        }
      }
    }
  }

  // 5b. coarse-space structure (subdomain couplings of the permuted CSR)
  {
    std::vector<int32_t> sub_of(n);
    for (int s = 0; s < a.n_sub; ++s)
      for (int32_t i = a.sub_ptr[s]; i < a.sub_ptr[s + 1]; ++i) sub_of[i] = s;
    a.cptr.assign(a.n_sub + 1, 0);
    a.cnb.clear();
    a.cslot.assign(a.nnz, 0);
    a.max_cnb = 0;
    std::vector<int32_t> nb;
    for (int s = 0; s < a.n_sub; ++s) {
      nb.clear();
      const int32_t e0 = a.prp[a.sub_ptr[s]], e1 = a.prp[a.sub_ptr[s + 1]];
      for (int32_t k = e0; k < e1; ++k) nb.push_back(sub_of[a.pci[k]]);
      std::sort(nb.begin(), nb.end());
      nb.erase(std::unique(nb.begin(), nb.end()), nb.end());
      a.max_cnb = std::max(a.max_cnb, (int)nb.size());
      if ((int)nb.size() <= kMaxCoarseNb)
        for (int32_t k = e0; k < e1; ++k)
          a.cslot[k] = (uint8_t)(std::lower_bound(nb.begin(), nb.end(),
                                                  sub_of[a.pci[k]]) -
                                 nb.begin());
      a.cnb.insert(a.cnb.end(), nb.begin(), nb.end());
      a.cptr[s + 1] = (int32_t)a.cnb.size();
    }
    // A Z per row (deflated coarse correction): the subdomains of the row's
    // columns, ascending, and each entry's position among them
    a.azp.assign(n + 1, 0);
    a.azj.clear();
    a.azslot.assign(a.nnz, 0);
    std::vector<int32_t> rs;
    for (int64_t i = 0; i < n; ++i) {
      rs.clear();
      for (int32_t k = a.prp[i]; k < a.prp[i + 1]; ++k) rs.push_back(sub_of[a.pci[k]]);
      std::sort(rs.begin(), rs.end());
      rs.erase(std::unique(rs.begin(), rs.end()), rs.end());
      for (int32_t k = a.prp[i]; k < a.prp[i + 1]; ++k)
        a.azslot[k] = (uint8_t)(std::lower_bound(rs.begin(), rs.end(),
                                                 sub_of[a.pci[k]]) - rs.begin());
      a.azj.insert(a.azj.end(), rs.begin(), rs.end());
      a.azp[i + 1] = (int32_t)a.azj.size();
    }
  }

  // 6. ILU(0) storage: the entries of each row inside its subdomain,
  //    L (columns before the row), diagonal, U (columns after)
  a.lrp.assign(n + 1, 0);
  a.ldg.assign(n, -1);
  a.lci.clear();
  a.lsrc.clear();
  std::vector<std::pair<int32_t, int32_t>> frow;  // (permuted col, entry)
  for (int s = 0; s < a.n_sub; ++s) {
    const int32_t r0 = a.sub_ptr[s], r1 = a.sub_ptr[s + 1];
    const int64_t e0 = (int64_t)a.lci.size();
    for (int32_t i = r0; i < r1 && fill > 0; ++i) {
      // ILU(k): the filled pattern, each entry with its permuted-CSR source
      // (-1 for fill, which starts at zero)
      frow.clear();
      for (int32_t c : fill_cols[a.perm[i]]) frow.push_back({a.iperm[c], -1});
      std::sort(frow.begin(), frow.end());
      for (int32_t k = a.prp[i]; k < a.prp[i + 1]; ++k) {
        auto it = std::lower_bound(frow.begin(), frow.end(),
                                   std::make_pair(a.pci[k], INT32_MIN));
        if (it != frow.end() && it->first == a.pci[k]) it->second = k;
      }
      for (const auto &e : frow) {
        if (e.first == i) a.ldg[i] = (int32_t)a.lci.size();
        a.lci.push_back(e.first - r0);
        a.lsrc.push_back(e.second);
      }
      a.lrp[i + 1] = (int32_t)a.lci.size();
    }
    for (int32_t i = r0; i < r1 && fill == 0; ++i) {
      bool have_diag = false;
      for (int32_t k = a.prp[i]; k < a.prp[i + 1]; ++k) {
        const int32_t c = a.pci[k];
        if (c < r0 || c >= r1) continue;
        if (c == i) {
          a.ldg[i] = (int32_t)a.lci.size();
          have_diag = true;
        } else if (c > i && !have_diag) {  // structural zero diagonal
          a.ldg[i] = (int32_t)a.lci.size();
          a.lci.push_back(i - r0);
          a.lsrc.push_back(-1);
          have_diag = true;
        }
        a.lci.push_back(c - r0);
        a.lsrc.push_back(k);
      }
      if (!have_diag) {
        a.ldg[i] = (int32_t)a.lci.size();
        a.lci.push_back(i - r0);
        a.lsrc.push_back(-1);
      }
      a.lrp[i + 1] = (int32_t)a.lci.size();
    }
    a.max_sub_lu = std::max(a.max_sub_lu, (int)((int64_t)a.lci.size() - e0));
  }

  // 7. packed per-subdomain records (layout in kernels.cuh): level bounds,
  //    then slot-major L/U column slots (subdomain-local, uint16) and value
  //    slots, so consecutive rows of a level sit in consecutive addresses;
  //    records and their sections start on 16-byte boundaries for
  //    cp.async.bulk
  PG_CHECK_ARG(a.max_sub_rows <= 65534,
               "ILU(0) subdomains are limited to 65534 rows (use Schwarz "
               "subdomains for larger systems)");
  auto al16 = [](int64_t b) { return (b + 15) & ~(int64_t)15; };
  a.meta64.resize(a.n_sub);
  int64_t off64 = 0, slots = 0;
  a.max_kl = a.max_ku = 0;
  for (int s = 0; s < a.n_sub; ++s) {
    const int32_t r0 = a.sub_ptr[s], r1 = a.sub_ptr[s + 1], nr = r1 - r0;
    int kl = 0, ku = 0;
    for (int32_t i = r0; i < r1; ++i) {
      kl = std::max(kl, a.ldg[i] - a.lrp[i]);
      ku = std::max(ku, a.lrp[i + 1] - a.ldg[i] - 1);
    }
    a.max_kl = std::max(a.max_kl, kl);
    a.max_ku = std::max(a.max_ku, ku);
    const int K = kl + ku;
    const int nlev = a.sub_lvl[s + 1] - a.sub_lvl[s];
    // lvl[] carries one sentinel past the last level bound
    const int64_t col_off = al16(2 * (int64_t)(nlev + 2));
    const int64_t val_off = col_off + al16(2 * (int64_t)nr * K);
    const int64_t bytes = val_off + al16(8 * (int64_t)nr * (K + 1));
    PG_CHECK_ARG(off64 + bytes < ((int64_t)1 << 31), "ILU(0) records too large");
    a.meta64[s] = SubMeta{r0, nr, nlev, K, kl, (int32_t)off64, (int32_t)col_off,
                          (int32_t)val_off, (int32_t)bytes, (int32_t)slots, 0, 0};
    off64 += bytes;
    slots += (int64_t)nr * (K + 1);
  }
  PG_CHECK_ARG(slots < ((int64_t)1 << 31), "ILU(0) factor too large");
  a.rec64.assign(off64, 0);
  a.rec_src.assign(slots, -1);
  a.smem64 = 0;
  for (int s = 0; s < a.n_sub; ++s) {
    const SubMeta &m = a.meta64[s];
    const int K = m.K, kl = m.KL, nr = m.nr;
    {
      const SubMeta &mm = m;
      uint8_t *base = a.rec64.data() + mm.rec_off;
      uint16_t *lvl = reinterpret_cast<uint16_t *>(base);
      for (int l = 0; l <= m.nlev; ++l)
        lvl[l] = (uint16_t)(a.lvl_ptr[a.sub_lvl[s] + l] - m.r0);
      lvl[m.nlev + 1] = (uint16_t)nr;
      uint16_t *cols = reinterpret_cast<uint16_t *>(base + mm.col_off);
      for (int i = 0; i < nr; ++i) {
        const int32_t g = m.r0 + i;
        const int nl = a.ldg[g] - a.lrp[g], nu = a.lrp[g + 1] - a.ldg[g] - 1;
        for (int k = 0; k < K; ++k) cols[(int64_t)k * nr + i] = kPadCol;
        for (int k = 0; k < nl; ++k)
          cols[(int64_t)k * nr + i] = (uint16_t)a.lci[a.lrp[g] + k];
        for (int k = 0; k < nu; ++k)
          cols[(int64_t)(kl + k) * nr + i] = (uint16_t)a.lci[a.ldg[g] + 1 + k];
        int32_t *src = a.rec_src.data() + m.slot_base;
        for (int k = 0; k < nl; ++k) src[(int64_t)k * nr + i] = a.lsrc[a.lrp[g] + k];
        for (int k = 0; k < nu; ++k)
          src[(int64_t)(kl + k) * nr + i] = a.lsrc[a.ldg[g] + 1 + k];
        src[(int64_t)K * nr + i] = a.lsrc[a.ldg[g]];
      }
      a.smem64 = std::max(a.smem64, (size_t)al16(mm.rec_bytes) + (size_t)nr * 8);
    }
  }

  // 8. streaming records (kernels.cuh StreamMeta): per level, the L slots
  //    (forward sweep) and the U slots + 1/u_ii (backward sweep) of the
  //    level's rows, slot-major; consecutive levels are grouped into pieces
  //    of about kStreamPiece bytes.  pack_* map every value position of a
  //    stream to its slot in the FP64 factor records.
  //    A record is a sweep group: one subdomain, or two consecutive ones
  //    whose levels fit side by side in one warp (every level of the pair
  //    at most 32 rows wide together); the group's level l holds level l of
  //    each member, so one warp sweeps both independent blocks at once.
  //    Pairs are formed only for single systems with compile-time slot
  //    counts (at most 3 L and 3 U entries per row).
  a.smeta64.clear();
  a.pack_src.clear();
  a.pack_dst64.clear();
  a.ssmem64 = 0;
  int64_t soff = 0;
  a.srec64.clear();
  // one slot count for all subdomains, matching the apply kernel's
  // compile-time variants (2/2 quadrilaterals, 3/3 triangles)
  int KLs = a.max_kl, KUs = a.max_ku;
  if (KLs <= 2 && KUs <= 2) KLs = KUs = 2;
  else if (KLs <= 3 && KUs <= 3) KLs = KUs = 3;
  const bool may_pair = !sys_rows && KLs <= 3 && KUs <= 3;
  auto lvl_of = [&](int s) {
    const SubMeta &f = a.meta64[s];
    return reinterpret_cast<const uint16_t *>(a.rec64.data() + f.rec_off);
  };
  auto width = [&](int s, int l) {
    const uint16_t *lv = lvl_of(s);
    return l < a.meta64[s].nlev ? lv[l + 1] - lv[l] : 0;
  };
  auto pairs_fit = [&](int s) {
    if (!may_pair || s + 1 >= a.n_sub) return false;
    if (a.meta64[s].nr + a.meta64[s + 1].nr + 1 > 65535) return false;
    const int nl = std::max(a.meta64[s].nlev, a.meta64[s + 1].nlev);
    for (int l = 0; l < nl; ++l)
      if (width(s, l) + width(s + 1, l) > 32) return false;
    return true;
  };
  for (int s = 0; s < a.n_sub;) {
    const int G = pairs_fit(s) ? 2 : 1;
    const SubMeta *mf[2] = {&a.meta64[s], G == 2 ? &a.meta64[s + 1] : nullptr};
    const int nr = mf[0]->nr + (G == 2 ? mf[1]->nr : 0);
    const int nlev = std::max(mf[0]->nlev, G == 2 ? mf[1]->nlev : 0);
    const int base[2] = {0, mf[0]->nr};
    const int KL = KLs, KU = KUs;
    // group level l: member m's rows [a_m, a_m + w_m) (group-local)
    auto lev = [&](int l, int m, int &am, int &wm) {
      wm = 0;
      am = base[m];
      if (m >= G) return;
      const uint16_t *lv = lvl_of(s + m);
      if (l < mf[m]->nlev) {
        am = base[m] + lv[l];
        wm = lv[l + 1] - lv[l];
      }
    };
    auto gw = [&](int l) {
      int a0, w0, a1, w1;
      lev(l, 0, a0, w0);
      lev(l, 1, a1, w1);
      return w0 + w1;
    };
    {
      const int64_t vs = 8;
      auto fblob = [&](int w) { return al16(2 * (int64_t)KL * w) + al16(vs * (int64_t)KL * w); };
      auto bblob = [&](int w) {
        return al16(2 * (int64_t)KU * w) + al16(vs * (int64_t)KU * w) + al16(vs * (int64_t)w);
      };
      // pieces: {first level, bytes}
      std::vector<std::pair<int, int64_t>> fp, bp;
      for (int l = 0; l < nlev; ++l) {
        const int64_t sz = fblob(gw(l));
        if (fp.empty() || fp.back().second + sz > kStreamPiece) fp.push_back({l, 0});
        fp.back().second += sz;
      }
      for (int l = nlev - 1; l >= 0; --l) {
        const int64_t sz = bblob(gw(l));
        if (bp.empty() || bp.back().second + sz > kStreamPiece) bp.push_back({l, 0});
        bp.back().second += sz;
      }
      for (auto &q : fp) q.second = std::max<int64_t>(q.second, 16);
      for (auto &q : bp) q.second = std::max<int64_t>(q.second, 16);
      const int np = (int)(fp.size() + bp.size());
      const int64_t lvl_bytes = 8 * (int64_t)nlev;  // 4 uint16 per level
      const int64_t hdr = al16(lvl_bytes + 4 * (2 + 3 * (int64_t)np));
      int64_t total = hdr, max_piece = 16;
      for (auto &q : fp) total += q.second, max_piece = std::max(max_piece, q.second);
      for (auto &q : bp) total += q.second, max_piece = std::max(max_piece, q.second);
      PG_CHECK_ARG(soff + total < ((int64_t)1 << 31), "ILU(0) stream too large");
      StreamMeta sm{};
      sm.r0 = mf[0]->r0;
      sm.nr = nr;
      sm.nlev = nlev;
      sm.KL = KL;
      sm.KU = KU;
      sm.rec_off = (int32_t)soff;
      sm.hdr_bytes = (int32_t)hdr;
      sm.max_piece = (int32_t)max_piece;
      sm.sub0 = s;
      sm.nsub = G;
      sm.nr0 = mf[0]->nr;
      std::vector<uint8_t> &buf = a.srec64;
      buf.resize(soff + total, 0);
      uint8_t *recb = buf.data() + soff;
      uint16_t *hl = reinterpret_cast<uint16_t *>(recb);
      for (int l = 0; l < nlev; ++l) {
        int a0, w0, a1, w1;
        lev(l, 0, a0, w0);
        lev(l, 1, a1, w1);
        hl[4 * l] = (uint16_t)a0;
        hl[4 * l + 1] = (uint16_t)w0;
        hl[4 * l + 2] = (uint16_t)a1;
        hl[4 * l + 3] = (uint16_t)w1;
      }
      int32_t *ints = reinterpret_cast<int32_t *>(recb + lvl_bytes);
      ints[0] = (int32_t)fp.size();
      ints[1] = (int32_t)bp.size();
      int64_t off = hdr;
      auto emit_values = [&](int m, int64_t byte_off, int64_t slot) {
        // byte_off is relative to this record; slot indexes member m's
        // factor record
        const int64_t fsrc0 = (mf[m]->rec_off + mf[m]->val_off) / 8;
        a.pack_src.push_back((int32_t)(fsrc0 + slot));
        a.pack_dst64.push_back((int32_t)((soff + byte_off) / vs));
      };
      // lane t of a group level: member m and its member-local row
      auto lane_row = [&](int l, int t, int &m, int &row) {
        int a0, w0, a1, w1;
        lev(l, 0, a0, w0);
        lev(l, 1, a1, w1);
        m = t < w0 ? 0 : 1;
        row = (m == 0 ? a0 + t : a1 + (t - w0)) - base[m];
      };
      auto emit_level = [&](int l, bool fwd) {
        const int w = gw(l);
        const int KS = fwd ? KL : KU;
        uint16_t *cc = reinterpret_cast<uint16_t *>(recb + off);
        const int64_t voff = off + al16(2 * (int64_t)KS * w);
        const int64_t doff = voff + al16(vs * (int64_t)KS * w);
        for (int k = 0; k < KS; ++k)
          for (int t = 0; t < w; ++t) {
            int m, row;
            lane_row(l, t, m, row);
            const SubMeta &f = *mf[m];
            const int fKL = f.KL, fKU = f.K - f.KL;
            const uint16_t *fcols = reinterpret_cast<const uint16_t *>(
                a.rec64.data() + f.rec_off + f.col_off);
            const int kk = fwd ? k : fKL + k;
            const bool used = fwd ? k < fKL : k < fKU;
            const int64_t slot = (int64_t)kk * f.nr + row;
            const uint16_t col = used ? fcols[slot] : kPadCol;
            // an unused slot points at the zero entry z[nr]
            cc[k * w + t] = col == kPadCol ? (uint16_t)nr : (uint16_t)(col + base[m]);
            if (col != kPadCol) emit_values(m, voff + vs * ((int64_t)k * w + t), slot);
          }
        if (!fwd)
          for (int t = 0; t < w; ++t) {
            int m, row;
            lane_row(l, t, m, row);
            const SubMeta &f = *mf[m];
            emit_values(m, doff + vs * t, (int64_t)f.K * f.nr + row);
          }
        off += fwd ? fblob(w) : bblob(w);
      };
      int t = 0;
      for (size_t q = 0; q < fp.size(); ++q, ++t) {
        const int l0 = fp[q].first;
        const int l1 = q + 1 < fp.size() ? fp[q + 1].first : nlev;
        ints[2 + 3 * t] = l0;
        ints[3 + 3 * t] = (int32_t)off;
        ints[4 + 3 * t] = (int32_t)fp[q].second;
        for (int l = l0; l < l1; ++l) emit_level(l, true);
      }
      for (size_t q = 0; q < bp.size(); ++q, ++t) {
        const int lhi = bp[q].first;
        const int llo = q + 1 < bp.size() ? bp[q + 1].first + 1 : 0;
        ints[2 + 3 * t] = lhi;
        ints[3 + 3 * t] = (int32_t)off;
        ints[4 + 3 * t] = (int32_t)bp[q].second;
        for (int l = lhi; l >= llo; --l) emit_level(l, false);
      }
      sm.p0_off = ints[3];
      sm.p0_bytes = ints[4];
      if (np > 1) {
        sm.p1_off = ints[6];
        sm.p1_bytes = ints[7];
      }
      a.smeta64.push_back(sm);
      soff += total;
      const size_t need = (size_t)hdr + 2 * (size_t)max_piece + (size_t)al16(vs * (int64_t)(nr + 1));
      a.ssmem64 = std::max(a.ssmem64, need);
    }
    s += G;
  }
  a.n_grp = (int)a.smeta64.size();

  // 8b. line form (kernels.cuh LineMeta) when every subdomain is a grid
  //     block: consecutive blocks of at most 16 lines are paired into one
  //     warp, other blocks of at most 32 lines take a warp each.  A group's
  //     record is [map][forward weights][backward weights]: map[r] is the
  //     line-major position (member offset + line * length + position) of
  //     the group's level-order row r, and the weights are stored line by
  //     line in that order (2 per row forward, 3 backward: the grid
  //     neighbours' weights and 1/u_ii), so lane i reads its own line's
  //     weights one after another.  pack_l* map every weight to its slot in
  //     the FP64 factor records.
  a.lmeta.clear();
  a.lrec.clear();
  a.lpack_src.clear();
  a.lpack_dst.clear();
  a.lsmem = 0;
  a.lmeta32.clear();
  a.lrec32.clear();
  a.lpack32_src.clear();
  a.lpack32_dst.clear();
  a.lsmem32 = 0;
  bool all_lines = want_line && a.n_sub > 0;
  for (int s = 0; s < a.n_sub && all_lines; ++s)
    all_lines = sub_lines[s] > 0 && sub_lines[s] <= 32 &&
                a.meta64[s].nlev <= 255 &&
                a.meta64[s].nr % sub_lines[s] == 0;
  // level-major records for 8-byte weights (k_ilu0_apply_line_lv): a
  // header of per-level member tables, then level blobs of weights in
  // pieces of about `piece` bytes streamed through shared memory
  auto build_lines_lv = [&](int64_t vs, int64_t piece, std::vector<LineMeta> &lmeta,
                         std::vector<uint8_t> &lrec,
                         std::vector<int32_t> &lpack_src,
                         std::vector<int32_t> &lpack_dst, size_t &lsmem) -> int {
    int64_t loff = 0;
    for (int s = 0; s < a.n_sub;) {
      const bool pair = s + 1 < a.n_sub && sub_lines[s] <= 16 &&
                        sub_lines[s + 1] <= 16 &&
                        a.meta64[s].nr + a.meta64[s + 1].nr < 65535;
      const int G = pair ? 2 : 1;
      const SubMeta *mf[2] = {&a.meta64[s], pair ? &a.meta64[s + 1] : nullptr};
      const int nr = mf[0]->nr + (pair ? mf[1]->nr : 0);
      const int nlev = std::max(mf[0]->nlev, pair ? mf[1]->nlev : 0);
      const int base[2] = {0, mf[0]->nr};
      // member m's rows of level l: group-local start, count, first line
      auto lev = [&](int l, int m, int &am, int &wm, int &lom) {
        am = base[m];
        wm = 0;
        lom = 0;
        if (m >= G || l >= mf[m]->nlev) return;
        const int32_t *lp = a.lvl_ptr.data() + a.sub_lvl[s + m];
        am = base[m] + (lp[l] - mf[m]->r0);
        wm = lp[l + 1] - lp[l];
        lom = gline[a.perm[lp[l]]];
      };
      auto wsum = [&](int l) {
        int am, w0, w1, lo;
        lev(l, 0, am, w0, lo);
        lev(l, 1, am, w1, lo);
        return w0 + w1;
      };
      auto fblob = [&](int w) { return al16(2 * vs * w); };
      auto bblob = [&](int w) { return al16(3 * vs * w); };
      std::vector<std::pair<int, int64_t>> fp, bp;
      for (int l = 0; l < nlev; ++l) {
        const int64_t sz = fblob(wsum(l));
        if (fp.empty() || fp.back().second + sz > piece) fp.push_back({l, 0});
        fp.back().second += sz;
      }
      for (int l = nlev - 1; l >= 0; --l) {
        const int64_t sz = bblob(wsum(l));
        if (bp.empty() || bp.back().second + sz > piece) bp.push_back({l, 0});
        bp.back().second += sz;
      }
      for (auto &q : fp) q.second = std::max<int64_t>(q.second, 16);
      for (auto &q : bp) q.second = std::max<int64_t>(q.second, 16);
      const int np = (int)(fp.size() + bp.size());
      const int64_t hdr = al16(8 * (int64_t)nlev + 4 * (2 + 3 * (int64_t)np));
      int64_t total = hdr, max_piece = 16;
      for (auto &q : fp) total += q.second, max_piece = std::max(max_piece, q.second);
      for (auto &q : bp) total += q.second, max_piece = std::max(max_piece, q.second);
      PG_CHECK_ARG(loff + total < ((int64_t)1 << 31), "ILU(0) line records too large");
      lrec.resize(loff + total, 0);
      uint8_t *recb = lrec.data() + loff;
      for (int l = 0; l < nlev; ++l) {
        int a0, w0, lo0, a1, w1, lo1;
        lev(l, 0, a0, w0, lo0);
        lev(l, 1, a1, w1, lo1);
        uint16_t *h16 = reinterpret_cast<uint16_t *>(recb + 8 * l);
        h16[0] = (uint16_t)a0;
        h16[1] = (uint16_t)a1;
        uint8_t *h8 = recb + 8 * l + 4;
        h8[0] = (uint8_t)w0;
        h8[1] = (uint8_t)lo0;
        h8[2] = (uint8_t)w1;
        h8[3] = (uint8_t)lo1;
      }
      int32_t *ints = reinterpret_cast<int32_t *>(recb + 8 * nlev);
      ints[0] = (int32_t)fp.size();
      ints[1] = (int32_t)bp.size();
      // the weight of the grid neighbour (line + dl, pos + dp) of member m's
      // factor row `row`: its slot in the factor record, or -1
      auto nb_slot = [&](int m, int row, bool lower, int dl, int dp) -> int64_t {
        const SubMeta &f = *mf[m];
        const int fKL = f.KL, fKU = f.K - f.KL;
        const uint16_t *fcols = reinterpret_cast<const uint16_t *>(
            a.rec64.data() + f.rec_off + f.col_off);
        const int32_t g = a.perm[f.r0 + row];
        const int k0 = lower ? 0 : fKL, kn = lower ? fKL : fKU;
        for (int k = 0; k < kn; ++k) {
          const int64_t sl = (int64_t)(k0 + k) * f.nr + row;
          if (fcols[sl] == kPadCol) continue;
          const int32_t c = a.perm[f.r0 + fcols[sl]];
          if (gline[c] == gline[g] + dl && gpos[c] == gpos[g] + dp) return sl;
        }
        return -1;
      };
      auto emit = [&](int m, int64_t byte_off, int64_t sl) {
        if (sl < 0) return;  // weight stays 0
        const int64_t fsrc0 = (mf[m]->rec_off + mf[m]->val_off) / 8;
        lpack_src.push_back((int32_t)(fsrc0 + sl));
        lpack_dst.push_back((int32_t)((loff + byte_off) / vs));
      };
      int64_t off = hdr;
      auto emit_level = [&](int l, bool fwd) {
        int am[2], wm[2], lom[2];
        lev(l, 0, am[0], wm[0], lom[0]);
        lev(l, 1, am[1], wm[1], lom[1]);
        int t = 0;
        for (int m = 0; m < 2; ++m)
          for (int k = 0; k < wm[m]; ++k, ++t) {
            const int row = am[m] - base[m] + k;  // member-local row
            if (fwd) {
              emit(m, off + vs * (2 * t), nb_slot(m, row, true, -1, 0));
              emit(m, off + vs * (2 * t + 1), nb_slot(m, row, true, 0, -1));
            } else {
              emit(m, off + vs * (3 * t), nb_slot(m, row, false, 1, 0));
              emit(m, off + vs * (3 * t + 1), nb_slot(m, row, false, 0, 1));
              emit(m, off + vs * (3 * t + 2),
                   (int64_t)mf[m]->K * mf[m]->nr + row);
            }
          }
        off += fwd ? fblob(t) : bblob(t);
      };
      int tq = 0;
      for (size_t q = 0; q < fp.size(); ++q, ++tq) {
        const int l0 = fp[q].first;
        const int l1 = q + 1 < fp.size() ? fp[q + 1].first : nlev;
        ints[2 + 3 * tq] = l0;
        ints[3 + 3 * tq] = (int32_t)off;
        ints[4 + 3 * tq] = (int32_t)fp[q].second;
        for (int l = l0; l < l1; ++l) emit_level(l, true);
      }
      for (size_t q = 0; q < bp.size(); ++q, ++tq) {
        const int lhi = bp[q].first;
        const int llo = q + 1 < bp.size() ? bp[q + 1].first + 1 : 0;
        ints[2 + 3 * tq] = lhi;
        ints[3 + 3 * tq] = (int32_t)off;
        ints[4 + 3 * tq] = (int32_t)bp[q].second;
        for (int l = lhi; l >= llo; --l) emit_level(l, false);
      }
      LineMeta lm{};
      lm.r0 = mf[0]->r0;
      lm.nr = nr;
      lm.nlev = nlev;
      lm.rec_off = (int32_t)loff;
      lm.hdr_bytes = (int32_t)hdr;
      lm.max_piece = (int32_t)max_piece;
      lm.p0_off = ints[3];
      lm.p0_bytes = ints[4];
      if (np > 1) {
        lm.p1_off = ints[6];
        lm.p1_bytes = ints[7];
      }
      lm.sub0 = s;
      lm.nsub = G;
      lm.nr0 = mf[0]->nr;
      lm.lanes = pair ? 16 : 32;
      // buffer 1 follows buffer 0; with two pieces each takes its own size
      lm.buf1 = np == 2 ? (int32_t)al16(ints[4]) : (int32_t)max_piece;
      lm.zs_off = (int32_t)(hdr + lm.buf1 + (np == 2 ? al16(ints[7]) : max_piece));
      lmeta.push_back(lm);
      loff += total;
      lsmem = std::max(lsmem, (size_t)lm.zs_off +
                                  (size_t)al16(8 * (int64_t)(nr + 1)));
      s += G;
    }
    return PG_OK;
  };
  // line-major records for FP32 weights (k_ilu0_apply_line)
  auto build_lines = [&](int64_t vs, std::vector<LineMeta> &lmeta,
                         std::vector<uint8_t> &lrec,
                         std::vector<int32_t> &lpack_src,
                         std::vector<int32_t> &lpack_dst, size_t &lsmem) -> int {
    int64_t loff = 0;
    for (int s = 0; s < a.n_sub;) {
      const bool pair = s + 1 < a.n_sub && sub_lines[s] <= 16 &&
                        sub_lines[s + 1] <= 16 &&
                        a.meta64[s].nr + a.meta64[s + 1].nr < 65535;
      const int G = pair ? 2 : 1;
      const SubMeta *mf[2] = {&a.meta64[s], pair ? &a.meta64[s + 1] : nullptr};
      const int nr = mf[0]->nr + (pair ? mf[1]->nr : 0);
      const int base[2] = {0, mf[0]->nr};
      int lines[2] = {0, 0}, len[2] = {0, 0}, nlev = 0;
      for (int m = 0; m < G; ++m) {
        lines[m] = sub_lines[s + m];
        len[m] = mf[m]->nr / lines[m];
        nlev = std::max(nlev, lines[m] + len[m] - 1);
      }
      const int64_t map_bytes = al16(2 * (int64_t)nr);
      const int64_t fw_bytes = al16(2 * vs * nr), bw_bytes = al16(3 * vs * nr);
      const int64_t total = map_bytes + fw_bytes + bw_bytes;
      PG_CHECK_ARG(loff + total < ((int64_t)1 << 31), "ILU(0) line records too large");
      lrec.resize(loff + total, 0);
      uint16_t *map = reinterpret_cast<uint16_t *>(lrec.data() + loff);
      // the weight of the grid neighbour (line + dl, pos + dp) of member m's
      // factor row `row`: its slot in the factor record, or -1
      auto nb_slot = [&](int m, int row, bool lower, int dl, int dp) -> int64_t {
        const SubMeta &f = *mf[m];
        const int fKL = f.KL, fKU = f.K - f.KL;
        const uint16_t *fcols = reinterpret_cast<const uint16_t *>(
            a.rec64.data() + f.rec_off + f.col_off);
        const int32_t g = a.perm[f.r0 + row];
        const int k0 = lower ? 0 : fKL, kn = lower ? fKL : fKU;
        for (int k = 0; k < kn; ++k) {
          const int64_t sl = (int64_t)(k0 + k) * f.nr + row;
          if (fcols[sl] == kPadCol) continue;
          const int32_t c = a.perm[f.r0 + fcols[sl]];
          if (gline[c] == gline[g] + dl && gpos[c] == gpos[g] + dp) return sl;
        }
        return -1;
      };
      auto emit = [&](int m, int64_t byte_off, int64_t sl) {
        if (sl < 0) return;  // weight stays 0
        const int64_t fsrc0 = (mf[m]->rec_off + mf[m]->val_off) / 8;
        lpack_src.push_back((int32_t)(fsrc0 + sl));
        lpack_dst.push_back((int32_t)((loff + byte_off) / vs));
      };
      for (int m = 0; m < G; ++m)
        for (int row = 0; row < mf[m]->nr; ++row) {
          const int32_t g = a.perm[mf[m]->r0 + row];
          PG_CHECK_ARG(gline[g] >= 0 && gline[g] < lines[m] && gpos[g] >= 0 &&
                           gpos[g] < len[m],
                       "line form: a row outside its block's grid");
          const int ln = base[m] + gline[g] * len[m] + gpos[g];
          map[base[m] + row] = (uint16_t)ln;
          const int64_t fo = map_bytes + vs * 2 * (int64_t)ln;
          emit(m, fo, nb_slot(m, row, true, -1, 0));
          emit(m, fo + vs, nb_slot(m, row, true, 0, -1));
          const int64_t bo = map_bytes + fw_bytes + vs * 3 * (int64_t)ln;
          emit(m, bo, nb_slot(m, row, false, 1, 0));
          emit(m, bo + vs, nb_slot(m, row, false, 0, 1));
          emit(m, bo + 2 * vs, (int64_t)mf[m]->K * mf[m]->nr + row);
        }
      LineMeta lm{};
      lm.r0 = mf[0]->r0;
      lm.nr = nr;
      lm.nlev = nlev;
      lm.rec_off = (int32_t)loff;
      lm.hdr_bytes = (int32_t)map_bytes;
      lm.max_piece = (int32_t)std::max(fw_bytes, bw_bytes);
      lm.p0_off = (int32_t)map_bytes;
      lm.p0_bytes = (int32_t)fw_bytes;
      lm.p1_off = (int32_t)(map_bytes + fw_bytes);
      lm.p1_bytes = (int32_t)bw_bytes;
      lm.sub0 = s;
      lm.nsub = G;
      lm.nr0 = mf[0]->nr;
      lm.lanes = pair ? 16 : 32;
      lm.buf1 = (int32_t)fw_bytes;
      lm.zs_off = (int32_t)(map_bytes + fw_bytes + bw_bytes);
      lm.lines0 = (int16_t)lines[0];
      lm.lines1 = (int16_t)lines[1];
      lm.len0 = (uint16_t)len[0];
      lm.len1 = (uint16_t)len[1];
      lmeta.push_back(lm);
      loff += total;
      // the group's vector (line-major)
      lsmem = std::max(lsmem, (size_t)lm.zs_off +
                                  (size_t)al16(8 * (int64_t)(nr + 1)));
      s += G;
    }
    return PG_OK;
  };
  if (all_lines) {
    int rc = build_lines_lv(8, 8192, a.lmeta, a.lrec, a.lpack_src, a.lpack_dst,
                            a.lsmem);
    if (!rc)
      rc = build_lines(4, a.lmeta32, a.lrec32, a.lpack32_src, a.lpack32_dst,
                       a.lsmem32);
    if (rc) return rc;
  }

  // 9. step stream for the float-float sweep of the mixed-precision solver
  //    (kernels.cuh StepMeta), when no row has more than 3 L or 3 U
  //    entries: warp-wide slices of a level with byte offsets into the
  //    subdomain's 8-byte z entries and {w0, w1, w2, 1/u_ii} as float pairs
  a.use_steps = a.max_kl <= 3 && a.max_ku <= 3 && a.max_sub_rows < 32767;
  a.tmeta_dd.clear();
  a.pack_src_dd.clear();
  a.pack_dst_dd.clear();
  a.srec_dd.clear();
  a.ssmem_dd = 0;
  if (a.use_steps) {
    constexpr int64_t es = 8;  // bytes of a z entry and of a float pair
    constexpr int64_t sb = kStepIdxBytes + 32 * 4 * es;
    a.tmeta_dd.resize(a.n_sub);
    int64_t toff = 0;
    for (int s = 0; s < a.n_sub; ++s) {
      const SubMeta &f = a.meta64[s];
      const int nr = f.nr, nlev = f.nlev, fKL = f.KL, fKU = f.K - f.KL;
      const int64_t fsrc0 = (f.rec_off + f.val_off) / 8;
      const uint16_t *flvl = reinterpret_cast<const uint16_t *>(a.rec64.data() + f.rec_off);
      const uint16_t *fcols =
          reinterpret_cast<const uint16_t *>(a.rec64.data() + f.rec_off + f.col_off);
      int n_fwd = 0;
      for (int l = 0; l < nlev; ++l) n_fwd += (flvl[l + 1] - flvl[l] + 31) / 32;
      const int n_bwd = n_fwd;
      const int64_t bytes = (int64_t)(n_fwd + n_bwd) * sb;
      PG_CHECK_ARG(toff + bytes < ((int64_t)1 << 31), "ILU(0) steps too large");
      a.tmeta_dd[s] = StepMeta{f.r0, nr, n_fwd, n_bwd, (int32_t)toff, 0, 0, 0};
      a.srec_dd.resize(toff + bytes, 0);
      uint8_t *base = a.srec_dd.data() + toff;
      int64_t step = 0;
      auto emit = [&](int64_t byte_off, int64_t slot) {
        a.pack_src_dd.push_back((int32_t)(fsrc0 + slot));
        a.pack_dst_dd.push_back((int32_t)((toff + byte_off) / es));
      };
      for (int dir = 0; dir < 2; ++dir) {
        const int k0 = dir == 0 ? 0 : fKL, kn = dir == 0 ? fKL : fKU;
        for (int li = 0; li < nlev; ++li) {
          const int l = dir == 0 ? li : nlev - 1 - li;
          for (int c0 = flvl[l]; c0 < flvl[l + 1]; c0 += 32, ++step) {
            uint32_t *idx = reinterpret_cast<uint32_t *>(base + step * sb);
            const uint32_t pad = (uint32_t)(nr * es);  // z[nr] == 0
            for (int t = 0; t < 32; ++t) {
              const int row = c0 + t;
              uint32_t *e = idx + 4 * t;
              e[0] = e[1] = e[2] = e[3] = pad;
              if (row >= flvl[l + 1]) continue;
              e[0] = (uint32_t)(row * es);
              for (int k = 0; k < kn; ++k) {
                const int64_t slot = (int64_t)(k0 + k) * nr + row;
                if (fcols[slot] == kPadCol) continue;
                e[1 + k] = (uint32_t)(fcols[slot] * es);
                emit(step * sb + kStepIdxBytes + es * (4 * t + k), slot);
              }
              if (dir == 1)
                emit(step * sb + kStepIdxBytes + es * (4 * t + 3),
                     (int64_t)(fKL + fKU) * nr + row);
            }
          }
        }
      }
      toff += bytes;
      const size_t need = 2 * (size_t)kStepsPerPiece * sb +
                          (size_t)al16(es * (int64_t)(nr + 1));
      a.ssmem_dd = std::max(a.ssmem_dd, need);
    }
  }
  return PG_OK;
}

}  // namespace pg
