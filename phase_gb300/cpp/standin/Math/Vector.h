// Stand-in for the parts of Phase's src/Math/Vector.h (Vector.h:8-42) the
// plugin touches: a dense vector of Scalars with data() and size().
#pragma once
#include <vector>
#include "Types/Types.h"
class Vector {
 public:
  explicit Vector(Size n = 0, Scalar v = 0.) : data_(n, v) {}
  Scalar &operator()(Index i) { return data_[i]; }
  Scalar operator()(Index i) const { return data_[i]; }
  size_t size() const { return data_.size(); }
  const std::vector<Scalar> &data() const { return data_; }
 private:
  std::vector<Scalar> data_;
};
