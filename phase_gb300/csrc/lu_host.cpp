// Symbolic analysis of the multifrontal sparse LU that stands in for
// Phase's direct backend, EigenSparseMatrixSolver (src/Math/
// EigenSparseMatrixSolver.cpp:5-64: setFromTriplets over the entries with
// col >= 0, duplicates summed; SparseLU compute + solve on every call).
//
// Ordering: nested dissection of the symmetrised pattern (George 1973).  A
// vertex set is cut in two halves (coordinate bisection across its longer
// extent when the rows carry points, e.g. cell centres; otherwise a
// breadth-first level structure from a pseudo-peripheral vertex split at
// its middle), the separator is the smaller of the two sides' boundary
// sets, the halves are dissected recursively and the separator is
// numbered after them.  A set of at most `leaf` vertices is not cut.
// Every node of the resulting tree is one front of the multifrontal method
// (Duff & Reid 1983; Liu, SIAM Review 34, 1992): its fully summed
// variables are its separator (or leaf set), its update variables the
// later-numbered vertices that its subtree couples to, which by the
// separator property are all ancestors.  The structure is computed for the
// symmetrised pattern, so it holds for the nonsymmetric ghost-cell rows as
// well.
#include <algorithm>
#include <cmath>
#include <numeric>

#include "internal.h"
#include "lu.h"

namespace pg {
namespace {

struct NdBuilder {
  int64_t n;
  const std::vector<int64_t> &ap;
  const std::vector<int32_t> &aj;
  const double *x, *y;
  int leaf;
  std::vector<int32_t> side;   // -1 outside the current set, 0 / 1 halves
  std::vector<int32_t> seen;
  int32_t stamp = 0;
  // nodes in creation (post) order
  std::vector<std::vector<int32_t>> sep;
  std::vector<std::vector<int32_t>> kids;

  NdBuilder(int64_t n_, const std::vector<int64_t> &ap_,
            const std::vector<int32_t> &aj_, const double *x_,
            const double *y_, int leaf_)
      : n(n_), ap(ap_), aj(aj_), x(x_), y(y_), leaf(leaf_), side(n_, -1),
        seen(n_, 0) {}

  int32_t make_node(std::vector<int32_t> s, std::vector<int32_t> ch) {
    std::sort(s.begin(), s.end());
    sep.push_back(std::move(s));
    kids.push_back(std::move(ch));
    return (int32_t)sep.size() - 1;
  }

  // breadth-first order of `v` (restarting at unvisited vertices so
  // disconnected sets are covered), from start; returns the visit order
  std::vector<int32_t> bfs(const std::vector<int32_t> &v, int32_t start) {
    ++stamp;
    std::vector<int32_t> q;
    q.reserve(v.size());
    size_t head = 0, scan = 0;
    q.push_back(start);
    seen[start] = stamp;
    while (q.size() < v.size()) {
      while (head < q.size()) {
        const int32_t u = q[head++];
        for (int64_t e = ap[u]; e < ap[u + 1]; ++e) {
          const int32_t w = aj[e];
          if (side[w] >= 0 && seen[w] != stamp) {
            seen[w] = stamp;
            q.push_back(w);
          }
        }
      }
      while (q.size() < v.size() && seen[v[scan]] == stamp) ++scan;
      if (q.size() < v.size()) {
        seen[v[scan]] = stamp;
        q.push_back(v[scan]);
      }
    }
    return q;
  }

  // roots of the dissection of v (several when the set falls apart)
  std::vector<int32_t> build(std::vector<int32_t> v) {
    if ((int64_t)v.size() <= leaf) {
      if (v.empty()) return {};
      return {make_node(std::move(v), {})};
    }
    for (int32_t u : v) side[u] = 0;
    const size_t half = v.size() / 2;
    if (x && y) {
      double x0 = INFINITY, x1 = -INFINITY, y0 = INFINITY, y1 = -INFINITY;
      for (int32_t u : v) {
        x0 = std::min(x0, x[u]);
        x1 = std::max(x1, x[u]);
        y0 = std::min(y0, y[u]);
        y1 = std::max(y1, y[u]);
      }
      const double *c = (x1 - x0 >= y1 - y0) ? x : y;
      // ties broken by index so the cut is deterministic
      std::nth_element(v.begin(), v.begin() + half, v.end(),
                       [c](int32_t a, int32_t b) {
                         return c[a] < c[b] || (c[a] == c[b] && a < b);
                       });
    } else {
      // pseudo-peripheral start: two sweeps from the smallest index
      int32_t s = *std::min_element(v.begin(), v.end());
      std::vector<int32_t> q = bfs(v, s);
      q = bfs(v, q.back());
      v.swap(q);
    }
    for (size_t i = 0; i < v.size(); ++i) side[v[i]] = i < half ? 0 : 1;
    std::vector<int32_t> sa, sb;
    for (size_t i = 0; i < v.size(); ++i) {
      const int32_t u = v[i];
      const int32_t su = side[u];
      bool cut = false;
      for (int64_t e = ap[u]; e < ap[u + 1] && !cut; ++e) {
        const int32_t w = aj[e];
        cut = side[w] >= 0 && side[w] != su;
      }
      if (cut) (su == 0 ? sa : sb).push_back(u);
    }
    std::vector<int32_t> &s = sa.size() <= sb.size() ? sa : sb;
    for (int32_t u : s) side[u] = 2;  // separator
    std::vector<int32_t> a, b;
    for (int32_t u : v) {
      if (side[u] == 0) a.push_back(u);
      else if (side[u] == 1) b.push_back(u);
    }
    for (int32_t u : v) side[u] = -1;
    std::vector<int32_t> sv(s.begin(), s.end());
    std::vector<int32_t> ra = build(std::move(a));
    std::vector<int32_t> rb = build(std::move(b));
    ra.insert(ra.end(), rb.begin(), rb.end());
    if (sv.empty()) return ra;  // the halves do not touch: a forest
    return {make_node(std::move(sv), std::move(ra))};
  }
};

}  // namespace

int lu_analyse(int64_t n, const int32_t *row_ptr, const int32_t *col_ind,
               const double *x, const double *y, int leaf, LuSymbolic &s) {
  PG_CHECK_ARG(n > 0 && row_ptr && col_ind, "lu_analyse: empty matrix");
  PG_CHECK_ARG(n < ((int64_t)1 << 31), "lu_analyse: rank too large");
  PG_CHECK_ARG(row_ptr[0] == 0, "row_ptr[0] must be 0");
  for (int64_t i = 0; i < n; ++i)
    PG_CHECK_ARG(row_ptr[i + 1] >= row_ptr[i], "row_ptr must be non-decreasing");
  const int64_t n_src = row_ptr[n];
  for (int64_t k = 0; k < n_src; ++k)
    PG_CHECK_ARG(col_ind[k] < n, "column index out of range");
  if (leaf <= 0) leaf = 64;
  s = LuSymbolic();
  s.n = n;
  s.n_src = n_src;

  // symmetrised adjacency without the diagonal
  std::vector<int64_t> ap(n + 1, 0);
  std::vector<int32_t> aj;
  {
    std::vector<int64_t> deg(n, 0);
    for (int64_t i = 0; i < n; ++i)
      for (int64_t k = row_ptr[i]; k < row_ptr[i + 1]; ++k) {
        const int32_t c = col_ind[k];
        if (c >= 0 && c != i) {
          ++deg[i];
          ++deg[c];
        }
      }
    for (int64_t i = 0; i < n; ++i) ap[i + 1] = ap[i] + deg[i];
    aj.resize(ap[n]);
    std::vector<int64_t> pos(ap.begin(), ap.end() - 1);
    for (int64_t i = 0; i < n; ++i)
      for (int64_t k = row_ptr[i]; k < row_ptr[i + 1]; ++k) {
        const int32_t c = col_ind[k];
        if (c >= 0 && c != i) {
          aj[pos[i]++] = c;
          aj[pos[c]++] = (int32_t)i;
        }
      }
    std::vector<int64_t> np(n + 1, 0);
    int64_t w = 0;
    for (int64_t i = 0; i < n; ++i) {
      std::sort(aj.begin() + ap[i], aj.begin() + ap[i + 1]);
      const int64_t e =
          std::unique(aj.begin() + ap[i], aj.begin() + ap[i + 1]) - aj.begin();
      for (int64_t k = ap[i]; k < e; ++k) aj[w++] = aj[k];
      np[i + 1] = w;
    }
    aj.resize(w);
    ap.swap(np);
  }

  // nested dissection
  NdBuilder nd(n, ap, aj, x, y, leaf);
  {
    std::vector<int32_t> all(n);
    std::iota(all.begin(), all.end(), 0);
    nd.build(std::move(all));
  }
  const int nf = (int)nd.sep.size();
  s.perm.resize(n);
  s.iperm.resize(n);
  s.fronts.resize(nf);
  std::vector<int32_t> node_of(n);
  {
    int32_t next = 0;
    for (int t = 0; t < nf; ++t) {
      LuFront &f = s.fronts[t];
      f = LuFront{};
      f.s0 = next;
      f.k = (int32_t)nd.sep[t].size();
      f.parent = -1;
      for (int32_t u : nd.sep[t]) {
        s.perm[next] = u;
        s.iperm[u] = next;
        node_of[next] = t;
        ++next;
      }
    }
  }
  for (int t = 0; t < nf; ++t) {
    LuFront &f = s.fronts[t];
    f.child_ptr = (int32_t)s.children.size();
    f.n_child = (int32_t)nd.kids[t].size();
    for (int32_t c : nd.kids[t]) {
      s.children.push_back(c);
      s.fronts[c].parent = t;
    }
  }

  // update sets, bottom-up (children are created before their parents)
  std::vector<std::vector<int32_t>> U(nf);
  {
    std::vector<int32_t> mark(n, -1);
    for (int t = 0; t < nf; ++t) {
      LuFront &f = s.fronts[t];
      const int32_t last = f.s0 + f.k - 1;
      std::vector<int32_t> &u = U[t];
      auto add = [&](int32_t v) {
        if (v > last && mark[v] != t) {
          mark[v] = t;
          u.push_back(v);
        }
      };
      for (int32_t i = f.s0; i <= last; ++i) {
        const int32_t o = s.perm[i];
        for (int64_t e = ap[o]; e < ap[o + 1]; ++e) add(s.iperm[aj[e]]);
      }
      for (int c = 0; c < f.n_child; ++c)
        for (int32_t v : U[s.children[f.child_ptr + c]]) add(v);
      std::sort(u.begin(), u.end());
      f.m = f.k + (int32_t)u.size();
      f.idx = (int32_t)s.fidx.size();
      for (int32_t i = 0; i < f.k; ++i) s.fidx.push_back(f.s0 + i);
      s.fidx.insert(s.fidx.end(), u.begin(), u.end());
      f.large = f.m > kLuSmallM ? 1 : 0;
      s.max_m = std::max(s.max_m, f.m);
      s.max_k = std::max(s.max_k, f.k);
      const double k = f.k, r = f.m - f.k;
      s.flops += 2. / 3. * k * k * k + 2. * k * k * r + 2. * k * r * r;
      s.factor_nnz += (int64_t)f.k * f.k + 2 * (int64_t)f.k * (f.m - f.k);
    }
  }
  // position of a new index v in front t's list
  auto pos_in = [&](int t, int32_t v) -> int32_t {
    const LuFront &f = s.fronts[t];
    if (v >= f.s0 && v < f.s0 + f.k) return v - f.s0;
    const std::vector<int32_t> &u = U[t];
    auto it = std::lower_bound(u.begin(), u.end(), v);
    if (it == u.end() || *it != v) return -1;
    return f.k + (int32_t)(it - u.begin());
  };
  // child maps
  for (int t = 0; t < nf; ++t) {
    LuFront &f = s.fronts[t];
    f.rel_off = (int32_t)s.rel.size();
    f.inv_off = -1;
    if (f.parent < 0) continue;
    const LuFront &p = s.fronts[f.parent];
    for (int32_t v : U[t]) {
      const int32_t q = pos_in(f.parent, v);
      PG_CHECK_ARG(q >= 0, "lu_analyse: update set not in the parent front");
      s.rel.push_back(q);
    }
    if (p.m > kLuSmallM) {
      f.inv_off = (int32_t)s.inv.size();
      s.inv.resize(s.inv.size() + p.m, -1);
      for (size_t a = 0; a < U[t].size(); ++a)
        s.inv[f.inv_off + s.rel[f.rel_off + a]] = (int32_t)a;
    }
  }

  // original entries: (i, j) belongs to the front of the earlier of its two
  // variables; repeated (i, j) are one entry summed over its sources
  {
    struct Ent {
      int32_t front, pos, src;
    };
    std::vector<Ent> ents;
    ents.reserve(n_src);
    s.src_col.assign(n_src, -1);
    for (int64_t i = 0; i < n; ++i)
      for (int64_t k = row_ptr[i]; k < row_ptr[i + 1]; ++k) {
        const int32_t c = col_ind[k];
        if (c < 0) continue;
        const int32_t ni = s.iperm[i], nj = s.iperm[c];
        s.src_col[k] = nj;
        const int t = node_of[std::min(ni, nj)];
        const int32_t pi = pos_in(t, ni), pj = pos_in(t, nj);
        PG_CHECK_ARG(pi >= 0 && pj >= 0, "lu_analyse: entry outside its front");
        ents.push_back({t, pi * s.fronts[t].m + pj, (int32_t)k});
      }
    std::stable_sort(ents.begin(), ents.end(), [](const Ent &a, const Ent &b) {
      return a.front < b.front || (a.front == b.front && a.pos < b.pos);
    });
    std::vector<int32_t> ent_front;  // owner of each unique entry
    for (size_t e = 0; e < ents.size(); ++e) {
      const Ent &q = ents[e];
      if (e == 0 || q.front != ents[e - 1].front || q.pos != ents[e - 1].pos) {
        s.e_pos.push_back(q.pos);
        s.e_ptr.push_back((int32_t)s.e_src.size());
        ent_front.push_back(q.front);
      }
      s.e_src.push_back(q.src);
    }
    s.e_ptr.push_back((int32_t)s.e_src.size());
    // entries are sorted by front: each front's range
    const int32_t ne = (int32_t)s.e_pos.size();
    int32_t e = 0;
    for (int t = 0; t < nf; ++t) {
      s.fronts[t].ent_ptr = e;
      while (e < ne && ent_front[e] == t) ++e;
      s.fronts[t].ent_end = e;
    }
  }

  // subtree ranges (postorder: a subtree's indices are contiguous)
  for (int t = 0; t < nf; ++t) {
    LuFront &f = s.fronts[t];
    f.first = f.s0;
    for (int c = 0; c < f.n_child; ++c)
      f.first = std::min(f.first, s.fronts[s.children[f.child_ptr + c]].first);
  }

  // heights, storage, task lists
  std::vector<int32_t> height(nf, 0);
  for (int t = 0; t < nf; ++t) {
    const LuFront &f = s.fronts[t];
    for (int c = 0; c < f.n_child; ++c)
      height[t] = std::max(height[t], height[s.children[f.child_ptr + c]] + 1);
  }
  s.n_heights = nf ? *std::max_element(height.begin(), height.end()) + 1 : 0;
  const int H = s.n_heights;
  s.h_small_ptr.assign(H + 1, 0);
  s.h_large_ptr.assign(H + 1, 0);
  s.h_all_ptr.assign(H + 1, 0);
  s.h_maxm.assign(H, 0);
  s.h_rows_ptr.assign(H + 1, 0);
  for (int h = 0; h < H; ++h) {
    s.h_small_ptr[h] = (int32_t)s.h_small.size();
    s.h_large_ptr[h] = (int32_t)s.h_large.size();
    s.h_all_ptr[h] = (int32_t)s.h_all.size();
    s.h_rows_ptr[h] = (int32_t)s.large_rows.size() / 2;
    for (int t = 0; t < nf; ++t) {
      if (height[t] != h) continue;
      LuFront &f = s.fronts[t];
      f.off = s.pool;
      s.pool += (int64_t)f.m * f.m;
      f.coff = s.cpool;
      s.cpool += f.m - f.k;
      s.h_all.push_back(t);
      s.h_maxm[h] = std::max(s.h_maxm[h], f.m);
      if (f.large) {
        s.h_large.push_back(t);
        for (int32_t r = 0; r < f.m; ++r) {
          s.large_rows.push_back(t);
          s.large_rows.push_back(r);
        }
      } else {
        s.h_small.push_back(t);
      }
    }
  }
  s.h_small_ptr[H] = (int32_t)s.h_small.size();
  s.h_large_ptr[H] = (int32_t)s.h_large.size();
  s.h_all_ptr[H] = (int32_t)s.h_all.size();
  s.h_rows_ptr[H] = (int32_t)s.large_rows.size() / 2;
  for (int h = 0; h < H; ++h) {
    int maxk = 0;
    for (int i = s.h_large_ptr[h]; i < s.h_large_ptr[h + 1]; ++i)
      maxk = std::max(maxk, s.fronts[s.h_large[i]].k);
    for (int q = 0; q * kLuPanel < maxk; ++q) {
      LuSymbolic::PanelStep st{};
      st.height = h;
      st.panel = q;
      st.diag_ptr = (int)s.pt_diag.size();
      st.trsm_ptr = (int)s.pt_trsm.size() / 3;
      st.upd_ptr = (int)s.pt_upd.size() / 3;
      for (int i = s.h_large_ptr[h]; i < s.h_large_ptr[h + 1]; ++i) {
        const int t = s.h_large[i];
        const LuFront &f = s.fronts[t];
        const int c0 = q * kLuPanel;
        if (f.k <= c0) continue;
        const int b = std::min(kLuPanel, f.k - c0);
        const int rest = f.m - c0 - b;  // trailing rows and columns
        s.pt_diag.push_back(t);
        for (int j0 = 0; j0 < rest; j0 += kLuTrsmCols) {  // U12 tiles
          s.pt_trsm.push_back(t);
          s.pt_trsm.push_back(1);
          s.pt_trsm.push_back(j0);
        }
        for (int i0 = 0; i0 < rest; i0 += kLuUpd)
          for (int j0 = 0; j0 < rest; j0 += kLuUpd) {
            s.pt_upd.push_back(t);
            s.pt_upd.push_back(i0);
            s.pt_upd.push_back(j0);
          }
      }
      st.diag_end = (int)s.pt_diag.size();
      st.trsm_end = (int)s.pt_trsm.size() / 3;
      st.upd_end = (int)s.pt_upd.size() / 3;
      s.steps.push_back(st);
    }
  }
  return PG_OK;
}

}  // namespace pg
