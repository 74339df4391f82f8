#include "Gb300SparseMatrixSolver.h"

#include <algorithm>
#include <cctype>
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
}

Gb300SparseMatrixSolver::~Gb300SparseMatrixSolver() {
  if (solver_) pg_solver_destroy(solver_);
}

// The library solver is created at the first setRank after construction or
// setup, so a configuration is checked before any device work.
void Gb300SparseMatrixSolver::recreate() {
  if (solver_) pg_solver_destroy(solver_);
  solver_ = nullptr;
  check(pg_solver_create(&cfg_, &solver_), "Gb300SparseMatrixSolver");
}

SparseMatrixSolver::Type Gb300SparseMatrixSolver::type() const {
  return SparseMatrixSolver::GB300;
}

void Gb300SparseMatrixSolver::setRank(int rank) {
  if (!solver_) recreate();
  rank_ = rank;
  check(pg_solver_set_rank(solver_, rank), "setRank");
  if (rank > 0 && xy_.size() == 2 * (size_t)rank)
    check(pg_solver_set_row_coords(solver_, xy_.data()), "setRank");
}

void Gb300SparseMatrixSolver::setRowCoordinates(const std::vector<Scalar> &xy) {
  xy_ = xy;
  if (solver_ && rank_ > 0 && xy_.size() == 2 * (size_t)rank_)
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

void Gb300SparseMatrixSolver::setDeviceEquation(const pg_eqn *eqn) {
  int64_t n = 0;
  check(pg_eqn_sizes(eqn, &n, nullptr), "setDeviceEquation");
  if (!solver_ || rank_ != (int)n) setRank((int)n);
  check(pg_solver_set_eqn(solver_, eqn), "setDeviceEquation");
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

namespace {

std::string upper(std::string s) {
  for (auto &c : s) c = (char)std::toupper((unsigned char)c);
  return s;
}

[[noreturn]] void unsupported(const std::string &what) {
  throw Exception("Gb300SparseMatrixSolver", "setup", what);
}

}  // namespace

// The keys of TrilinosBelosSparseMatrixSolver::setup
// (src/Math/TrilinosBelosSparseMatrixSolver.cpp:44-86) with their defaults,
// plus this backend's own.  A value the backend does not build throws
// instead of being replaced by another method.
void Gb300SparseMatrixSolver::setup(const boost::property_tree::ptree &p) {
  pg_solver_default_cfg(&cfg_);
  cfg_.tolerance = p.get<Scalar>("tolerance", 1e-8);
  cfg_.max_iters = p.get<int>("maxIters", 500);
  if (!p.get<std::string>("belosParamFile", "").empty() ||
      !p.get<std::string>("ifpackParamFile", "").empty())
    unsupported("belosParamFile/ifpackParamFile (Teuchos XML parameter "
                "lists) are not read by lib gb300; give the keys directly.");
  const std::string solver = upper(p.get<std::string>("solver", "BICGSTAB"));
  if (solver == "BICGSTAB")
    cfg_.krylov = PG_KRYLOV_BICGSTAB;
  else if (solver == "TFQMR")
    cfg_.krylov = PG_KRYLOV_TFQMR;
  else if (solver == "GMRES")
    cfg_.krylov = PG_KRYLOV_GMRES;
  else
    unsupported("solver \"" + solver + "\" is not built (BICGSTAB, TFQMR, "
                "GMRES are).");
  cfg_.krylov_dim = p.get<int>("numBlocks", 0);
  // Without ifpackParamFile the reference always builds Ifpack2 "schwarz"
  // whatever "preconditioner" says (:63-67); "none" and "jacobi" are this
  // backend's own values.
  const std::string pre = upper(p.get<std::string>("preconditioner", "schwarz"));
  const std::string inner =
      upper(p.get<std::string>("innerPreconditioner", "RILUK"));
  if (pre == "NONE") {
    cfg_.precond = PG_PREC_NONE;
  } else if (pre == "JACOBI" || inner == "RELAXATION" || inner == "DIAGONAL") {
    // Schwarz over point-Jacobi blocks is point Jacobi (one sweep, no damping)
    cfg_.precond = PG_PREC_JACOBI;
  } else if (inner == "RILUK") {
    cfg_.precond = PG_PREC_ILU0;
  } else {
    unsupported("innerPreconditioner \"" + inner + "\" is not built "
                "(RILUK with iluFill k, RELAXATION and DIAGONAL are).");
  }
  const double fill = p.get<Scalar>("iluFill", 0.);
  if (!(fill >= 0.) || fill != (double)(int)fill)
    unsupported("iluFill must be a non-negative whole level of fill.");
  cfg_.ilu_fill = (int)fill;
  if (p.get<int>("schwarzIters", 1) != 1)
    unsupported("schwarzIters other than 1 is not built.");
  if (upper(p.get<std::string>("schwarzCombineMode", "ADD")) != "ADD")
    unsupported("schwarzCombineMode other than ADD is not built.");
  if (p.get<int>("schwarzOverlap", 0) != 0)
    unsupported("schwarzOverlap other than 0 is not built.");
  cfg_.subdomain_rows = p.get<int>("subdomainRows", 0);
  const std::string prec = upper(p.get<std::string>("precision", "fp64"));
  if (prec != "FP64" && prec != "MIXED")
    unsupported("precision must be fp64 or mixed.");
  cfg_.precision = prec == "MIXED" ? PG_MIXED : PG_FP64;
  cfg_.mixed_sweep = p.get<int>("mixedSweep", 0);
  // two-level by default: the plugin is selected for speed, and the
  // deflated coarse correction cuts pressure solves 20-30x in iterations;
  // coarseSpace 0 gives the one-level Schwarz of Ifpack2
  cfg_.coarse = p.get<int>("coarseSpace", 2);
  cfg_.coarse_warm = p.get<int>("coarseWarmIters", -1);
  if (solver_) pg_solver_destroy(solver_);
  solver_ = nullptr;  // created with this configuration at the next setRank
  rank_ = 0;
}

int Gb300SparseMatrixSolver::nIters() const { return stats_.iters; }

Scalar Gb300SparseMatrixSolver::error() const { return stats_.rel_residual; }

void Gb300SparseMatrixSolver::printStatus(const std::string &msg) const {
  std::printf("%s %s iterations = %d, error = %lf.\n", msg.c_str(), "Krylov",
              nIters(), error());
}
