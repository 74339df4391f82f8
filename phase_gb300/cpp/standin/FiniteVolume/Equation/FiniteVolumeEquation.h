// Stand-in for Phase's FiniteVolume/Equation/FiniteVolumeEquation.h as a
// GB300 build has it: FiniteVolumeEquation<Scalar> is the device equation
// of Gb300FiniteVolume.h, and that header's fv::laplacian / src::div
// overloads are in scope wherever the equation is.  Inside Phase the
// specialisation sits beside the generic template.
#pragma once
#include <string>

#include "FiniteVolume/Field/ScalarFiniteVolumeField.h"
#include "FiniteVolume/Field/VectorFiniteVolumeField.h"
#include "Gb300FiniteVolume.h"

template <class T> class FiniteVolumeEquation;

template <> class FiniteVolumeEquation<Scalar> : public gb300::DeviceScalarEquation {
 public:
  explicit FiniteVolumeEquation(ScalarFiniteVolumeField &field,
                                const std::string &name = "")
      : gb300::DeviceScalarEquation(field, name) {}
  using gb300::DeviceScalarEquation::operator=;
};
