// Drives Gb300SparseMatrixSolver exactly as FiniteVolumeEquation::solve does
// (setRank, set(rowPtr, colInd, vals) with CrsEquation's 5-slot layout and -1
// placeholders, setRhs(-rhs), solve, x(i)) on a 2D Poisson problem and
// checks the true residual.  Exit code 0 on success.
#include <cmath>
#include <cstdio>
#include <vector>

#include "Gb300SparseMatrixSolver.h"
#include "System/Exception.h"

int main() {
  const int nx = 40, ny = 30, n = nx * ny;
  std::vector<Index> rp(n + 1), ci(5 * n, -1);
  std::vector<Scalar> v(5 * n, 0.);
  for (int i = 0; i <= n; ++i) rp[i] = 5 * i;
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i) {
      int r = j * nx + i, k = 5 * r;
      double d = 0.;
      auto nb = [&](int c) { ci[k] = c; v[k++] = 1.; d -= 1.; };
      if (i > 0) nb(r - 1);
      if (i < nx - 1) nb(r + 1);
      if (j > 0) nb(r - nx);
      if (j < ny - 1) nb(r + nx);
      d -= 1.;  // Dirichlet-like sink keeps the system non-singular
      ci[k] = r;
      v[k] = d;
    }
  Vector b(n);
  for (int i = 0; i < n; ++i) b(i) = std::sin(0.1 * i);
  Gb300SparseMatrixSolver s;
  boost::property_tree::ptree p;
  p.put("tolerance", "1e-10");
  p.put("maxIters", "2000");
  s.setup(p);
  s.setRank(n);
  s.set(rp, ci, v);
  s.setRhs(b);
  s.solve();
  double rr = 0., bb = 0.;
  for (int r = 0; r < n; ++r) {
    double ax = 0.;
    for (int k = rp[r]; k < rp[r + 1]; ++k)
      if (ci[k] >= 0) ax += v[k] * s.x(ci[k]);
    rr += (b(r) - ax) * (b(r) - ax);
    bb += b(r) * b(r);
  }
  double rel = std::sqrt(rr / bb);
  s.printStatus("shim_test pEqn:");
  std::printf("true relative residual %.3e\n", rel);
  if (!(rel <= 1.01e-10) || s.error() > 1e-10 || s.nIters() <= 0) return 1;
  // a bad argument surfaces as a Phase Exception
  try {
    s.setRank(3);
    std::vector<Index> bad(2, 0);
    s.set(bad, ci, v);
    return 2;
  } catch (const Exception &e) {
    std::printf("exception as expected: %s\n", e.what());
  }
  return 0;
}
