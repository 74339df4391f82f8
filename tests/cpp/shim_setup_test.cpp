// Gb300SparseMatrixSolver::setup reads the Belos backend's keys
// (TrilinosBelosSparseMatrixSolver.cpp:44-86): values the backend builds are
// accepted, every other value throws Phase's Exception instead of being
// replaced by another method.  setup does no device work, so this runs
// without a GPU.  Exit code 0 on success, else the number of the failed case.
#include <cstdio>
#include <string>
#include <vector>

#include "Gb300SparseMatrixSolver.h"
#include "System/Exception.h"

namespace {

bool throws(const std::vector<std::pair<std::string, std::string>> &kv) {
  Gb300SparseMatrixSolver s;
  boost::property_tree::ptree p;
  for (const auto &e : kv) p.put(e.first, e.second);
  try {
    s.setup(p);
  } catch (const Exception &e) {
    std::printf("rejected: %s\n", e.what());
    return true;
  }
  return false;
}

}  // namespace

int main() {
  int failed = 0, k = 0;
  auto expect = [&](bool cond) {
    ++k;
    if (!cond && !failed) failed = k;
  };
  expect(!throws({}));
  expect(!throws({{"solver", "bicgstab"}, {"preconditioner", "DIAGONAL"}}));
  expect(!throws({{"solver", "TFQMR"}}));
  expect(!throws({{"solver", "GMRES"}, {"numBlocks", "50"}}));
  expect(!throws({{"innerPreconditioner", "RILUK"}, {"iluFill", "0"}}));
  expect(!throws({{"innerPreconditioner", "RELAXATION"}}));
  expect(!throws({{"schwarzOverlap", "0"}, {"schwarzCombineMode", "add"}}));
  expect(throws({{"solver", "CG"}}));
  expect(throws({{"innerPreconditioner", "ILUT"}}));
  expect(throws({{"iluFill", "0.5"}}));
  expect(throws({{"schwarzOverlap", "1"}}));
  expect(throws({{"schwarzCombineMode", "ZERO"}}));
  expect(throws({{"schwarzIters", "3"}}));
  expect(throws({{"belosParamFile", "belos.xml"}}));
  expect(throws({{"ifpackParamFile", "ifpack.xml"}}));
  expect(throws({{"precision", "fp16"}}));
  std::printf("%d cases, first failure %d\n", k, failed);
  return failed;
}
