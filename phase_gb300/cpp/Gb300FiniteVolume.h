// The pressure equation of Phase's fractional-step solvers assembled on the
// GB300 behind Phase's own fv:: / src:: expressions.
//
// FractionalStepMultiphase::solvePEqn writes
//     pEqn_ = (fv::laplacian(timeStep / rho_, p_) == src::div(u_));
//     Scalar error = pEqn_.solve();
// (src/2D/Unstructured/Solvers/FractionalStepMultiphase.cpp:152-156; the
// single-phase form with a scalar coefficient is FractionalStep.cpp:96-107).
// With this header in a GB300 build the same two statements, unchanged,
// assemble the CSR and its right-hand side on the device (the face-coloured
// kernels of pg_assemble_laplacian) and hand them to the GB300 solver with
// no host copy of the matrix (pg_solver_set_eqn):
//  * fv::laplacian(const ScalarFiniteVolumeField &gamma,
//    ScalarFiniteVolumeField &phi) and fv::laplacian(Scalar, ...) are
//    non-template overloads, so overload resolution prefers them to Phase's
//    function templates for the same arguments (Laplacian.h:49-83,132-167);
//    they return a LaplacianTerm that records its operands;
//  * src::div(const VectorFiniteVolumeField &u) returns a DivergenceSource
//    (the sums of Source.cpp:5-25, evaluated in the assembly kernels); in a
//    Phase tree this declaration takes the place of Source.h's (the one
//    line a GB300 build changes there);
//  * term == source is a PressureSystem (CrsEquation::operator==(Vector),
//    CrsEquation.cpp:309-311), which DeviceScalarEquation -- the
//    FiniteVolumeEquation<Scalar> of a GB300 build -- takes by assignment
//    and solves, writing the solution into the field's cells
//    (ScalarFiniteVolumeEquation.cpp:59-64).
// The grid is copied to the device once (pg_mesh_create numbers faces as
// FiniteVolumeGrid2D::init does, so face and cell ids agree); the device
// equation is rebuilt only when the field's boundary types change.
// Errors surface as Phase's Exception.
#pragma once
#include <cstdint>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "Gb300SparseMatrixSolver.h"
#include "System/Exception.h"
#include "phase_gb300.h"

namespace gb300 {

inline void check(int rc, const char *what) {
  if (rc != PG_OK) throw Exception("gb300", what, pg_last_error());
}

// The device copy of a Phase grid, built on first use and kept for the
// life of the process (grids live as long as their solver).
template <class Grid>
pg_mesh *device_mesh(const Grid &grid) {
  static std::mutex mu;
  static std::map<const void *, pg_mesh *> meshes;
  std::lock_guard<std::mutex> lock(mu);
  auto it = meshes.find(&grid);
  if (it != meshes.end()) return it->second;
  std::vector<double> xy;
  xy.reserve(2 * grid.nodes().size());
  for (const auto &node : grid.nodes()) {
    xy.push_back(node.x);
    xy.push_back(node.y);
  }
  std::vector<int64_t> cptr(1, 0), cind;
  for (const auto &cell : grid.cells()) {
    for (const auto &node : cell.nodes()) cind.push_back((int64_t)node.get().id());
    cptr.push_back((int64_t)cind.size());
  }
  pg_mesh *m = nullptr;
  check(pg_mesh_create(xy.data(), (int64_t)grid.nodes().size(), cptr.data(),
                       cind.data(), (int64_t)grid.cells().size(), &m),
        "device_mesh");
  meshes[&grid] = m;
  return m;
}

// fv::laplacian(gamma, phi): face-field or scalar coefficient
struct LaplacianTerm {
  const ScalarFiniteVolumeField *gamma = nullptr;  // NULL: gamma_scalar
  Scalar gamma_scalar = 0.;
  ScalarFiniteVolumeField *phi = nullptr;
};

// src::div(u): the face velocities whose outward fluxes make the source
struct DivergenceSource {
  const VectorFiniteVolumeField *u = nullptr;
};

// fv::laplacian(gamma, phi) == src::div(u)
struct PressureSystem {
  LaplacianTerm lap;
  const VectorFiniteVolumeField *u = nullptr;
};

inline PressureSystem operator==(const LaplacianTerm &lap,
                                 const DivergenceSource &div) {
  return PressureSystem{lap, div.u};
}

// FiniteVolumeEquation<Scalar> of a GB300 build: the equation lives on the
// device; solve() runs the GB300 solver configured from the case's
// LinearAlgebra.<name> keys (Gb300SparseMatrixSolver::setup).
class DeviceScalarEquation {
 public:
  explicit DeviceScalarEquation(ScalarFiniteVolumeField &field,
                                const std::string &name = "")
      : field_(&field), name_(name),
        solver_(std::make_shared<Gb300SparseMatrixSolver>()) {}
  DeviceScalarEquation(const DeviceScalarEquation &) = delete;
  DeviceScalarEquation &operator=(const DeviceScalarEquation &) = delete;
  ~DeviceScalarEquation() {
    if (eqn_) pg_eqn_destroy(eqn_);
  }

  // LinearAlgebra.<name> (FiniteVolumeEquation::configureSparseSolver,
  // FiniteVolumeEquation.tpp:47-62)
  void configureSparseSolver(const boost::property_tree::ptree &keys) {
    solver_->setup(keys);
  }

  // assembles fv::laplacian(gamma, phi) == src::div(u) on the device
  DeviceScalarEquation &operator=(const PressureSystem &sys) {
    const ScalarFiniteVolumeField &phi = *sys.lap.phi;
    const auto &grid = *phi.grid();
    pg_mesh *m = device_mesh(grid);
    const int kind = sys.lap.gamma ? PG_GAMMA_FACE : PG_GAMMA_SCALAR;
    std::vector<int32_t> bc(grid.faces().size(), PG_BC_NORMAL_GRADIENT);
    for (const auto &face : grid.faces()) {
      if (!face.isBoundary()) continue;
      switch (phi.boundaryType(face)) {
        case ScalarFiniteVolumeField::FIXED: bc[face.id()] = PG_BC_FIXED; break;
        case ScalarFiniteVolumeField::NORMAL_GRADIENT:
          bc[face.id()] = PG_BC_NORMAL_GRADIENT;
          break;
        case ScalarFiniteVolumeField::SYMMETRY: bc[face.id()] = PG_BC_SYMMETRY; break;
        default:
          throw Exception("fv", "laplacian",
                          "unrecognized or unspecified boundary type.");
      }
    }
    if (!eqn_ || kind != kind_ || bc != bc_ || m != mesh_) {
      if (eqn_) pg_eqn_destroy(eqn_);
      eqn_ = nullptr;
      check(pg_eqn_create(m, kind, bc.data(), &eqn_), "laplacian");
      kind_ = kind;
      bc_ = bc;
      mesh_ = m;
    }
    std::vector<double> uf;
    if (sys.u) {
      const auto &faces = sys.u->faces();
      uf.resize(2 * faces.size());
      for (size_t f = 0; f < faces.size(); ++f) {
        uf[2 * f] = faces[f].x;
        uf[2 * f + 1] = faces[f].y;
      }
    }
    check(pg_assemble_laplacian(eqn_,
                                sys.lap.gamma ? sys.lap.gamma->faces().data() : nullptr,
                                sys.lap.gamma_scalar, phi.faces().data(),
                                sys.u ? uf.data() : nullptr, PG_HOST),
          "laplacian");
    field_ = sys.lap.phi;
    return *this;
  }

  // FiniteVolumeEquation<T>::solve (FiniteVolumeEquation.tpp:64-86): the
  // device matrix and -rhs_ to the solver, the solution to the cells
  Scalar solve() {
    if (!eqn_)
      throw Exception("FiniteVolumeEquation<T>", "solve",
                      "nothing has been assembled.");
    solver_->setDeviceEquation(eqn_);
    solver_->solve();
    const size_t n = field_->size();
    for (size_t i = 0; i < n; ++i) (*field_)[i] = solver_->x((Index)i);
    solver_->printStatus("FiniteVolumeEquation " + name_ + ":");
    return solver_->error();
  }

  int nIters() const { return solver_->nIters(); }
  const pg_eqn *deviceEquation() const { return eqn_; }

 private:
  ScalarFiniteVolumeField *field_;
  std::string name_;
  std::shared_ptr<Gb300SparseMatrixSolver> solver_;
  pg_eqn *eqn_ = nullptr;
  pg_mesh *mesh_ = nullptr;
  int kind_ = -1;
  std::vector<int32_t> bc_;
};

}  // namespace gb300

namespace fv {
// Laplacian.h:132-167 on the device
inline gb300::LaplacianTerm laplacian(const ScalarFiniteVolumeField &gamma,
                                      ScalarFiniteVolumeField &phi) {
  return gb300::LaplacianTerm{&gamma, 0., &phi};
}
// Laplacian.h:49-83 on the device
inline gb300::LaplacianTerm laplacian(Scalar gamma, ScalarFiniteVolumeField &phi) {
  return gb300::LaplacianTerm{nullptr, gamma, &phi};
}
}  // namespace fv

namespace src {
// Source.cpp:5-25 evaluated by the assembly kernels
inline gb300::DivergenceSource div(const VectorFiniteVolumeField &u) {
  return gb300::DivergenceSource{&u};
}
}  // namespace src
