// The GB300 direct backend for Phase: a drop-in for EigenSparseMatrixSolver
// (src/Math/EigenSparseMatrixSolver.{h,cpp}), the backend that
// SparseMatrixSolverFactory::create returns for `lib eigen` / `lib eigen3`
// (src/Math/SparseMatrixSolverFactory.cpp:26-40).  It keeps that class's
// behaviour -- the matrix of the entries with col >= 0 (repeated entries
// summed), a factorisation and solve on every solve() after new values,
// nIters() = 1, error() = 0, setGuess ignored -- and runs the
// factorisation and the triangular solves on the device through the C ABI
// (pg_lu_*, include/phase_gb300.h).
#pragma once
#include <vector>

#include "Math/SparseMatrixSolver.h"
#include "phase_gb300.h"

class Gb300SparseLUSolver : public SparseMatrixSolver {
 public:
  Gb300SparseLUSolver();
  ~Gb300SparseLUSolver() override;

  Type type() const override { return EIGEN; }
  void setRank(int rank) override;
  void setRank(int rowRank, int colRank) override;
  void set(const CoefficientList &coeffs) override;
  void set(const std::vector<Index> &rowPtr, const std::vector<Index> &colInds,
           const std::vector<Scalar> &vals) override;
  void set(const std::vector<SparseEntry> &entries) override;
  void setGuess(const Vector &x0) override {}
  void setRhs(const Vector &rhs) override;
  Scalar solve() override;
  Scalar x(Index idx) const override { return x_[idx]; }
  int nIters() const override { return 1; }
  Scalar error() const override { return 0.; }
  bool supportsMPI() const override { return false; }
  // Optional geometry hint (no EigenSparseMatrixSolver counterpart): a
  // point per row, xy[2 * rank] interleaved (the cell centroids), so the
  // nested-dissection ordering is cut by coordinates.
  void setRowCoordinates(const std::vector<Scalar> &xy);
  // The matrix and -rhs_ of an equation assembled on the device (the
  // device form of FiniteVolumeEquation::solve's setRank + set + setRhs,
  // FiniteVolumeEquation.tpp:71-73).
  void setDeviceEquation(const pg_eqn *eqn);
  // statistics of the last solve (fronts, flops, times, FP64 residual)
  const pg_lu_stats &stats() const { return stats_; }

 private:
  void check(int rc, const char *method) const;
  pg_lu *lu_ = nullptr;
  pg_lu_stats stats_{};
  int rank_ = 0;
  std::vector<Scalar> x_;
  std::vector<Scalar> xy_;
};
