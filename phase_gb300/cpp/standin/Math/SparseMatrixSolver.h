// Stand-in for Phase's src/Math/SparseMatrixSolver.h (:11-62): the same
// virtual interface, plus a GB300 enumerator that a Phase build adds next to
// EIGEN/TRILINOS_* when it registers this backend.  Inside Phase the real
// header is used.
#pragma once
#include <string>
#include <tuple>
#include <utility>
#include <vector>
#include <boost/property_tree/ptree.hpp>
#include "Math/SparseEntry.h"
#include "Math/Vector.h"
class SparseMatrixSolver {
 public:
  enum Type { EIGEN, TRILINOS_BELOS, TRILINOS_AMESOS2, TRILINOS_MUELU, GB300 };
  typedef std::pair<Index, Scalar> Entry;
  typedef std::vector<Entry> Row;
  typedef std::vector<Row> CoefficientList;
  virtual ~SparseMatrixSolver() = default;
  virtual Type type() const = 0;
  virtual void setRank(int rank) = 0;
  virtual void setRank(int rowRank, int colRank) = 0;
  virtual void set(const CoefficientList &eqn) = 0;
  virtual void set(const std::vector<Index> &rowPtr,
                   const std::vector<Index> &colInds,
                   const std::vector<Scalar> &vals) = 0;
  virtual void set(const std::vector<SparseEntry> &entries) = 0;
  virtual void setGuess(const Vector &x0) = 0;
  virtual void setRhs(const Vector &rhs) = 0;
  virtual Scalar solve() = 0;
  virtual Scalar x(Index idx) const = 0;
  virtual void setup(const boost::property_tree::ptree &parameters) {}
  virtual int nIters() const = 0;
  virtual Scalar error() const = 0;
  virtual bool supportsMPI() const = 0;
  virtual void printStatus(const std::string &msg) const {}
};
