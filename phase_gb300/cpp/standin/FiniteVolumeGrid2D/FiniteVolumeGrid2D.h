// Stand-in for the parts of Phase's FiniteVolumeGrid2D the device equation
// reads: nodes (coordinates, ids), cells (ids, nodes in order) and faces
// (ids, boundary flag), with faces numbered as FiniteVolumeGrid2D::init /
// createCell number them (FiniteVolumeGrid2D.cpp:84-114): cells in order,
// each cell's edges in order, a new face for every node pair not seen
// before.  Inside Phase the real header is used.
#pragma once
#include <algorithm>
#include <cstdint>
#include <functional>
#include <map>
#include <utility>
#include <vector>

#include "Geometry/Vector2D.h"
#include "Types/Types.h"

template <class T> using Ref = std::reference_wrapper<T>;

class Node : public Vector2D {
 public:
  Node(Scalar x, Scalar y, Label id) : Vector2D(x, y), id_(id) {}
  Label id() const { return id_; }
 private:
  Label id_;
};

class Cell {
 public:
  Cell(Label id, std::vector<Ref<const Node>> nodes)
      : id_(id), nodes_(std::move(nodes)) {}
  Label id() const { return id_; }
  const std::vector<Ref<const Node>> &nodes() const { return nodes_; }
 private:
  Label id_;
  std::vector<Ref<const Node>> nodes_;
};

class Face {
 public:
  Face(Label id, Label l) : id_(id), l_(l) {}
  Label id() const { return id_; }
  bool isBoundary() const { return !interior_; }
  bool isInterior() const { return interior_; }
  void setRight(Label r) { r_ = r, interior_ = true; }
 private:
  Label id_, l_, r_ = 0;
  bool interior_ = false;
};

class FiniteVolumeGrid2D {
 public:
  FiniteVolumeGrid2D(const std::vector<Scalar> &xy,
                     const std::vector<int64_t> &cptr,
                     const std::vector<int64_t> &cind) {
    nodes_.reserve(xy.size() / 2);
    for (size_t k = 0; 2 * k < xy.size(); ++k)
      nodes_.emplace_back(xy[2 * k], xy[2 * k + 1], (Label)k);
    std::map<std::pair<int64_t, int64_t>, Label> seen;
    for (size_t c = 0; c + 1 < cptr.size(); ++c) {
      std::vector<Ref<const Node>> nodes;
      for (int64_t k = cptr[c]; k < cptr[c + 1]; ++k)
        nodes.push_back(std::cref(nodes_[cind[k]]));
      cells_.emplace_back((Label)c, nodes);
      const int64_t m = cptr[c + 1] - cptr[c];
      for (int64_t k = 0; k < m; ++k) {
        const int64_t a = cind[cptr[c] + k], b = cind[cptr[c] + (k + 1) % m];
        const auto key = std::make_pair(std::min(a, b), std::max(a, b));
        auto it = seen.find(key);
        if (it == seen.end()) {
          seen[key] = (Label)faces_.size();
          faces_.emplace_back((Label)faces_.size(), (Label)c);
        } else {
          faces_[it->second].setRight((Label)c);
        }
      }
    }
  }
  const std::vector<Node> &nodes() const { return nodes_; }
  const std::vector<Cell> &cells() const { return cells_; }
  const std::vector<Face> &faces() const { return faces_; }
 private:
  std::vector<Node> nodes_;
  std::vector<Cell> cells_;
  std::vector<Face> faces_;
};
