// Stand-in for Phase's src/Math/SparseEntry.h (SparseEntry.h:6-16).
#pragma once
#include "Types/Types.h"
class SparseEntry {
 public:
  SparseEntry() {}
  SparseEntry(Index r, Index c, Scalar v) : row(r), col(c), val(v) {}
  Index row, col;
  Scalar val;
};
