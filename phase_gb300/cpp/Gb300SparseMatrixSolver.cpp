#include "Gb300SparseMatrixSolver.h"

#include <algorithm>
#include <cstdio>
#include <string>

#include "System/Exception.h"

// Status codes of the C ABI become Phase Exceptions (System/Exception.h);
// solver outcomes (max iterations, breakdown) are reported through
// error()/nIters() as the Belos backend does.
void Gb300SparseMatrixSolver::check(int rc, const char *method) const {
  if (rc == PG_OK || rc == PG_MAX_ITERS || rc == PG_BREAKDOWN) return;
  throw Exception("Gb300SparseMatrixSolver", method, pg_last_error());
}

Gb300SparseMatrixSolver::Gb300SparseMatrixSolver() {
  pg_solver_default_cfg(&cfg_);
  cfg_.coarse = 2;  // as setup() without a coarseSpace key
  recreate();
}

Gb300SparseMatrixSolver::~Gb300SparseMatrixSolver() {
  if (solver_) pg_solver_destroy(solver_);
}

void Gb300SparseMatrixSolver::recreate() {
  if (solver_) pg_solver_destroy(solver_);
  solver_ = nullptr;
  check(pg_solver_create(&cfg_, &solver_), "Gb300SparseMatrixSolver");
}

SparseMatrixSolver::Type Gb300SparseMatrixSolver::type() const {
  return SparseMatrixSolver::GB300;
}

void Gb300SparseMatrixSolver::setRank(int rank) {
  rank_ = rank;
  check(pg_solver_set_rank(solver_, rank), "setRank");
  if (rank > 0 && xy_.size() == 2 * (size_t)rank)
    check(pg_solver_set_row_coords(solver_, xy_.data()), "setRank");
}

void Gb300SparseMatrixSolver::setRowCoordinates(const std::vector<Scalar> &xy) {
  xy_ = xy;
  if (rank_ > 0 && xy_.size() == 2 * (size_t)rank_)
    check(pg_solver_set_row_coords(solver_, xy_.data()), "setRowCoordinates");
}

void Gb300SparseMatrixSolver::setRank(int rowRank, int colRank) {
  if (rowRank != colRank)
    throw Exception("Gb300SparseMatrixSolver", "setRank",
                    "rectangular systems are not supported.");
  setRank(rowRank);
}

void Gb300SparseMatrixSolver::set(const std::vector<Index> &rowPtr,
                                  const std::vector<Index> &colInds,
                                  const std::vector<Scalar> &vals) {
  if ((int)rowPtr.size() != rank_ + 1)
    throw Exception("Gb300SparseMatrixSolver", "set",
                    "rowPtr size does not match the rank.");
  check(pg_solver_set_csr(solver_, rowPtr.data(), colInds.data(), vals.data(),
                          PG_HOST),
        "set");
}

void Gb300SparseMatrixSolver::set(const CoefficientList &eqn) {
  std::vector<Index> rp(1, 0), ci;
  std::vector<Scalar> v;
  for (const auto &row : eqn) {
    for (const auto &e : row) {
      ci.push_back(e.first);
      v.push_back(e.second);
    }
    rp.push_back((Index)ci.size());
  }
  rp.resize(rank_ + 1, rp.back());
  set(rp, ci, v);
}

void Gb300SparseMatrixSolver::set(const std::vector<SparseEntry> &entries) {
  std::vector<SparseEntry> e(entries);
  std::stable_sort(e.begin(), e.end(), [](const SparseEntry &a,
                                          const SparseEntry &b) {
    return a.row < b.row;
  });
  std::vector<Index> rp(rank_ + 1, 0), ci;
  std::vector<Scalar> v;
  for (const auto &s : e) {
    if (s.row < 0 || s.row >= rank_)
      throw Exception("Gb300SparseMatrixSolver", "set", "row out of range.");
    ++rp[s.row + 1];
    ci.push_back(s.col);
    v.push_back(s.val);
  }
  for (int i = 0; i < rank_; ++i) rp[i + 1] += rp[i];
  set(rp, ci, v);
}

void Gb300SparseMatrixSolver::setGuess(const Vector &x0) {
  check(pg_solver_set_guess(solver_, x0.data().data(), PG_HOST), "setGuess");
}

void Gb300SparseMatrixSolver::setRhs(const Vector &rhs) {
  check(pg_solver_set_rhs(solver_, rhs.data().data(), PG_HOST), "setRhs");
}

Scalar Gb300SparseMatrixSolver::solve() {
  int rc = pg_solver_solve(solver_, &stats_);
  check(rc, "solve");
  x_.resize(rank_);
  check(pg_solver_get_x(solver_, x_.data(), PG_HOST), "solve");
  return error();
}

Scalar Gb300SparseMatrixSolver::x(Index idx) const { return x_[idx]; }

void Gb300SparseMatrixSolver::setup(const boost::property_tree::ptree &p) {
  cfg_.tolerance = p.get<Scalar>("tolerance", 1e-8);
  cfg_.max_iters = p.get<int>("maxIters", 500);
  const std::string pre = p.get<std::string>("preconditioner", "ilu0");
  cfg_.precond = pre == "none" ? PG_PREC_NONE
                 : pre == "jacobi" || pre == "diagonal" ? PG_PREC_JACOBI
                                                        : PG_PREC_ILU0;
  cfg_.subdomain_rows = p.get<int>("subdomainRows", 0);
  cfg_.precision =
      p.get<std::string>("precision", "fp64") == "mixed" ? PG_MIXED : PG_FP64;
  cfg_.mixed_sweep = p.get<int>("mixedSweep", 0);
  // two-level by default: the plugin is selected for speed, and the
  // deflated coarse correction cuts pressure solves 20-30x in iterations;
  // coarseSpace 0 gives the one-level Schwarz of Ifpack2
  cfg_.coarse = p.get<int>("coarseSpace", 2);
  cfg_.coarse_warm = p.get<int>("coarseWarmIters", -1);
  recreate();
}

int Gb300SparseMatrixSolver::nIters() const { return stats_.iters; }

Scalar Gb300SparseMatrixSolver::error() const { return stats_.rel_residual; }

void Gb300SparseMatrixSolver::printStatus(const std::string &msg) const {
  std::printf("%s %s iterations = %d, error = %lf.\n", msg.c_str(), "Krylov",
              nIters(), error());
}
