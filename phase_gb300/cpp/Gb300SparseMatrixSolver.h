// The GB300 SparseMatrixSolver plugin for Phase: registered in
// SparseMatrixSolverFactory::create (src/Math/SparseMatrixSolverFactory.cpp
// :26-40) as `lib gb300`, it replaces the Belos BiCGStab + Ifpack2 RILUK
// backend (src/Math/TrilinosBelosSparseMatrixSolver.cpp) by the CUDA solver
// of libphase_gb300 through its C ABI (include/phase_gb300.h).
#pragma once
#include <vector>

#include "Math/SparseMatrixSolver.h"
#include "phase_gb300.h"

class Gb300SparseMatrixSolver : public SparseMatrixSolver {
 public:
  Gb300SparseMatrixSolver();
  ~Gb300SparseMatrixSolver() override;

  Type type() const override;
  void setRank(int rank) override;
  void setRank(int rowRank, int colRank) override;
  void set(const CoefficientList &eqn) override;
  void set(const std::vector<Index> &rowPtr, const std::vector<Index> &colInds,
           const std::vector<Scalar> &vals) override;
  void set(const std::vector<SparseEntry> &entries) override;
  void setGuess(const Vector &x0) override;
  void setRhs(const Vector &rhs) override;
  Scalar solve() override;
  Scalar x(Index idx) const override;
  // keys of the Belos backend: tolerance (1e-8), maxIters (500), solver
  // (BICGSTAB | TFQMR | GMRES), innerPreconditioner (RILUK | RELAXATION |
  // DIAGONAL), iluFill (level of fill, 0), schwarzIters (1),
  // schwarzCombineMode (ADD), schwarzOverlap (0); preconditioner is
  // ignored as the reference does (always Schwarz) except this backend's
  // own values none and jacobi.  Own keys: numBlocks (GMRES restart length,
  // 300), subdomainRows (0 = default, -1 = one subdomain), precision (fp64
  // | mixed), mixedSweep (0 | 1 | 2), coarseSpace (2 default: deflated
  // two-level Schwarz; 1 additive; 0 one-level, as Ifpack2),
  // coarseWarmIters (-1 default).  Other values of the reference's keys,
  // and belosParamFile / ifpackParamFile, throw Exception.
  void setup(const boost::property_tree::ptree &parameters) override;
  // Optional geometry hint (no SparseMatrixSolver counterpart): a point per
  // row, xy[2 * rank] interleaved (the cell centroids), so the Schwarz
  // subdomains are cut by coordinate bisection.  Kept across setRank calls
  // of the same rank.
  void setRowCoordinates(const std::vector<Scalar> &xy);
  // The matrix and -rhs_ of an equation assembled on the device (the
  // device form of FiniteVolumeEquation::solve's setRank + set + setRhs,
  // FiniteVolumeEquation.tpp:71-73): no host copy of the CSR is made.
  void setDeviceEquation(const pg_eqn *eqn);
  int nIters() const override;
  Scalar error() const override;
  bool supportsMPI() const override { return false; }
  void printStatus(const std::string &msg) const override;

 private:
  void check(int rc, const char *method) const;
  void recreate();
  pg_solver *solver_ = nullptr;
  pg_solver_cfg cfg_;
  pg_solve_stats stats_{};
  int rank_ = 0;
  std::vector<Scalar> x_;
  std::vector<Scalar> xy_;  // setRowCoordinates
};
