// Drives Gb300SparseLUSolver exactly as FiniteVolumeEquation::solve drives
// EigenSparseMatrixSolver (setRank, set(rowPtr, colInd, vals) with
// CrsEquation's 5-slot layout and -1 placeholders, setRhs(-rhs), solve,
// x(i)) on a 2D Poisson problem, then the CoefficientList and triplet
// forms of set(); checks the true residual of each.  Exit code 0 on success.
#include <cmath>
#include <cstdio>
#include <vector>

#include "Gb300SparseLUSolver.h"
#include "System/Exception.h"

static double residual(const std::vector<Index> &rp, const std::vector<Index> &ci,
                       const std::vector<Scalar> &v, const Vector &b,
                       const SparseMatrixSolver &s) {
  double rr = 0., bb = 0.;
  const int n = (int)rp.size() - 1;
  for (int r = 0; r < n; ++r) {
    double ax = 0.;
    for (int k = rp[r]; k < rp[r + 1]; ++k)
      if (ci[k] >= 0) ax += v[k] * s.x(ci[k]);
    rr += (b(r) - ax) * (b(r) - ax);
    bb += b(r) * b(r);
  }
  return std::sqrt(rr / bb);
}

int main() {
  const int nx = 60, ny = 45, n = nx * ny;
  std::vector<Index> rp(n + 1), ci(5 * n, -1);
  std::vector<Scalar> v(5 * n, 0.);
  for (int i = 0; i <= n; ++i) rp[i] = 5 * i;
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i) {
      int r = j * nx + i, k = 5 * r;
      double d = 0.;
      const double w = 1.0 + 0.5 * std::sin(0.3 * i + 0.2 * j);
      auto nb = [&](int c) { ci[k] = c; v[k++] = w; d -= w; };
      if (i > 0) nb(r - 1);
      if (i < nx - 1) nb(r + 1);
      if (j > 0) nb(r - nx);
      if (j < ny - 1) nb(r + nx);
      d -= 0.5;
      ci[k] = r;
      v[k] = d;
    }
  Vector b(n);
  for (int i = 0; i < n; ++i) b(i) = std::sin(0.1 * i) + 0.25;
  Gb300SparseLUSolver s;
  boost::property_tree::ptree p;
  s.setup(p);
  s.setRank(n);
  s.set(rp, ci, v);
  s.setRhs(b);
  s.solve();
  const double rel = residual(rp, ci, v, b, s);
  std::printf("direct solve: true relative residual %.3e, %d fronts, "
              "factorisation %.3f ms\n", rel, s.stats().n_fronts,
              s.stats().factor_ms);
  if (!(rel <= 1e-12) || s.nIters() != 1 || s.error() != 0.) return 1;
  // the CoefficientList form of the same matrix
  SparseMatrixSolver::CoefficientList rows(n);
  for (int r = 0; r < n; ++r)
    for (int k = rp[r]; k < rp[r + 1]; ++k)
      if (ci[k] >= 0) rows[r].push_back({ci[k], v[k]});
  Gb300SparseLUSolver s2;
  s2.setRank(n);
  s2.set(rows);
  s2.setRhs(b);
  s2.solve();
  if (!(residual(rp, ci, v, b, s2) <= 1e-12)) return 2;
  for (int r = 0; r < n; ++r)
    if (s2.x(r) != s.x(r)) return 3;  // same pattern order: same factors
  // a bad argument surfaces as a Phase Exception
  try {
    s.setRank(3);
    std::vector<Index> bad(2, 0);
    s.set(bad, ci, v);
    return 4;
  } catch (const Exception &e) {
    std::printf("exception as expected: %s\n", e.what());
  }
  return 0;
}
