#include "Gb300SparseLUSolver.h"

#include <algorithm>

#include "System/Exception.h"

void Gb300SparseLUSolver::check(int rc, const char *method) const {
  if (rc != PG_OK) throw Exception("Gb300SparseLUSolver", method, pg_last_error());
}

Gb300SparseLUSolver::Gb300SparseLUSolver() {
  check(pg_lu_create(&lu_), "Gb300SparseLUSolver");
}

Gb300SparseLUSolver::~Gb300SparseLUSolver() {
  if (lu_) pg_lu_destroy(lu_);
}

// EigenSparseMatrixSolver::setRank (EigenSparseMatrixSolver.cpp:5-9)
void Gb300SparseLUSolver::setRank(int rank) {
  rank_ = rank;
  check(pg_lu_set_rank(lu_, rank), "setRank");
  if (rank > 0 && xy_.size() == 2 * (size_t)rank)
    check(pg_lu_set_row_coords(lu_, xy_.data()), "setRank");
}

// EigenSparseMatrixSolver::setRank(rowRank, colRank) (:11-15) sizes a
// rectangular matrix for SparseLU, which factorises square matrices only
void Gb300SparseLUSolver::setRank(int rowRank, int colRank) {
  if (rowRank != colRank)
    throw Exception("Gb300SparseLUSolver", "setRank",
                    "rectangular systems are not supported.");
  setRank(rowRank);
}

void Gb300SparseLUSolver::setRowCoordinates(const std::vector<Scalar> &xy) {
  xy_ = xy;
  if (rank_ > 0 && xy_.size() == 2 * (size_t)rank_)
    check(pg_lu_set_row_coords(lu_, xy_.data()), "setRowCoordinates");
}

// set(rowPtr, colInds, vals) (:31-40): col < 0 skipped, repeats summed
void Gb300SparseLUSolver::set(const std::vector<Index> &rowPtr,
                              const std::vector<Index> &colInds,
                              const std::vector<Scalar> &vals) {
  if ((int)rowPtr.size() != rank_ + 1)
    throw Exception("Gb300SparseLUSolver", "set",
                    "rowPtr size does not match the rank.");
  check(pg_lu_set_csr(lu_, rowPtr.data(), colInds.data(), vals.data(), PG_HOST),
        "set");
}

// set(CoefficientList) (:17-29): row i's (column, value) pairs
void Gb300SparseLUSolver::set(const CoefficientList &coeffs) {
  std::vector<Index> rp(1, 0), ci;
  std::vector<Scalar> v;
  for (const auto &row : coeffs) {
    for (const auto &e : row) {
      ci.push_back(e.first);
      v.push_back(e.second);
    }
    rp.push_back((Index)ci.size());
  }
  rp.resize(rank_ + 1, rp.back());
  set(rp, ci, v);
}

// set(vector<SparseEntry>) (:42-48): triplets, repeats summed
void Gb300SparseLUSolver::set(const std::vector<SparseEntry> &entries) {
  std::vector<SparseEntry> e(entries);
  std::stable_sort(e.begin(), e.end(), [](const SparseEntry &a,
                                          const SparseEntry &b) {
    return a.row < b.row;
  });
  std::vector<Index> rp(rank_ + 1, 0), ci;
  std::vector<Scalar> v;
  for (const auto &s : e) {
    if (s.row < 0 || s.row >= rank_)
      throw Exception("Gb300SparseLUSolver", "set", "row out of range.");
    ++rp[s.row + 1];
    ci.push_back(s.col);
    v.push_back(s.val);
  }
  for (int i = 0; i < rank_; ++i) rp[i + 1] += rp[i];
  set(rp, ci, v);
}

void Gb300SparseLUSolver::setDeviceEquation(const pg_eqn *eqn) {
  int64_t n = 0;
  check(pg_eqn_sizes(eqn, &n, nullptr), "setDeviceEquation");
  if (rank_ != (int)n) setRank((int)n);
  check(pg_lu_set_eqn(lu_, eqn), "setDeviceEquation");
}

// setRhs (:55-58)
void Gb300SparseLUSolver::setRhs(const Vector &rhs) {
  check(pg_lu_set_rhs(lu_, rhs.data().data(), PG_HOST), "setRhs");
}

// solve (:60-64): factorise (when the values changed) and solve
Scalar Gb300SparseLUSolver::solve() {
  check(pg_lu_solve(lu_, &stats_), "solve");
  x_.resize(rank_);
  check(pg_lu_get_x(lu_, x_.data(), PG_HOST), "solve");
  return 0.;
}
