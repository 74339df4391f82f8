// Stand-in for Phase's ScalarFiniteVolumeField and the operator/(Scalar,
// field) the pressure coefficient timeStep / rho uses
// (ScalarFiniteVolumeField.cpp:68-81: the quotient on cells and faces).
// Inside Phase the real header is used.
#pragma once
#include "FiniteVolume/Field/FiniteVolumeField.h"

class ScalarFiniteVolumeField : public FiniteVolumeField<Scalar> {
 public:
  using FiniteVolumeField<Scalar>::FiniteVolumeField;
};

inline ScalarFiniteVolumeField operator/(Scalar lhs, ScalarFiniteVolumeField rhs) {
  for (Scalar &v : rhs) v = lhs / v;
  for (Scalar &v : rhs.faces()) v = lhs / v;
  return rhs;
}
