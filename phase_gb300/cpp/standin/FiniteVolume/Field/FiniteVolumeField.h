// Stand-in for Phase's FiniteVolumeField<T>
// (src/2D/Unstructured/FiniteVolume/Field/FiniteVolumeField.h:12-190): cell
// values (the vector itself, by cell id), face values (faces(), by face
// id), a boundary type per boundary face and the grid.  Inside Phase the
// real header is used.
#pragma once
#include <memory>
#include <vector>

#include "FiniteVolumeGrid2D/FiniteVolumeGrid2D.h"

template <class T> class FiniteVolumeField : public std::vector<T> {
 public:
  enum BoundaryType { FIXED, NORMAL_GRADIENT, SYMMETRY, OUTFLOW, PARTIAL_SLIP };
  explicit FiniteVolumeField(const std::shared_ptr<const FiniteVolumeGrid2D> &grid,
                             const T &val = T())
      : std::vector<T>(grid->cells().size(), val),
        grid_(grid), faces_(grid->faces().size(), val),
        types_(grid->faces().size(), NORMAL_GRADIENT) {}
  const std::shared_ptr<const FiniteVolumeGrid2D> &grid() const { return grid_; }
  std::vector<T> &faces() { return faces_; }
  const std::vector<T> &faces() const { return faces_; }
  T &operator()(const Cell &cell) { return (*this)[cell.id()]; }
  const T &operator()(const Cell &cell) const { return (*this)[cell.id()]; }
  T &operator()(const Face &face) { return faces_[face.id()]; }
  const T &operator()(const Face &face) const { return faces_[face.id()]; }
  BoundaryType boundaryType(const Face &face) const { return types_[face.id()]; }
  void setBoundaryType(const Face &face, BoundaryType t) { types_[face.id()] = t; }
 private:
  std::shared_ptr<const FiniteVolumeGrid2D> grid_;
  std::vector<T> faces_;
  std::vector<BoundaryType> types_;
};
