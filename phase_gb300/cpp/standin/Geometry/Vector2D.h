// Stand-in for Phase's src/2D/Geometry/Vector2D.h (Vector2D.h:10-65): the
// two public components the device equation reads.  Inside Phase the real
// header is used.
#pragma once
#include "Types/Types.h"
class Vector2D {
 public:
  Vector2D(Scalar x = 0., Scalar y = 0.) : x(x), y(y) {}
  Scalar x, y;
};
