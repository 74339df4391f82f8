// Stand-in for Phase's VectorFiniteVolumeField (face velocities as
// Vector2D).  Inside Phase the real header is used.
#pragma once
#include "FiniteVolume/Field/FiniteVolumeField.h"

class VectorFiniteVolumeField : public FiniteVolumeField<Vector2D> {
 public:
  using FiniteVolumeField<Vector2D>::FiniteVolumeField;
};
