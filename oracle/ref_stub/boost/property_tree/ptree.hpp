// Stand-in for the one Boost type that src/Math/SparseMatrixSolver.h names
// (only in the signature of SparseMatrixSolver::setup).  It lets the
// reference's own CrsEquation.cpp, Vector.cpp and Exception.cpp compile
// without Boost so the oracle can be checked against them.  Test
// infrastructure only.
#pragma once
namespace boost {
namespace property_tree {
class ptree {};
}  // namespace property_tree
}  // namespace boost
