// Phase's pressure step through the GB300 fv:: drop-in: a
// FractionalStepMultiphase-shaped class whose solvePEqn holds the two
// statements of FractionalStepMultiphase::solvePEqn
// (src/2D/Unstructured/Solvers/FractionalStepMultiphase.cpp:152-156)
// unchanged, compiled against Phase-shaped stand-in field types and
// Gb300FiniteVolume.h.  Inputs (mesh, densities, face velocities, the
// pressure's boundary types and values) come from the file argv[1]; p on
// the cells, the solver's error and iterations go to argv[2].
#include <cstdint>
#include <cstdio>
#include <memory>
#include <vector>

#include "FiniteVolume/Equation/FiniteVolumeEquation.h"
#include "boost/property_tree/ptree.hpp"

class MultiphasePressureStep {
 public:
  explicit MultiphasePressureStep(const std::shared_ptr<const FiniteVolumeGrid2D> &g)
      : p_(g), rho_(g), u_(g), pEqn_(p_, "pEqn") {}

  Scalar solvePEqn(Scalar timeStep) {
    pEqn_ = (fv::laplacian(timeStep / rho_, p_) == src::div(u_));

    Scalar error = pEqn_.solve();
    return error;
  }

  ScalarFiniteVolumeField p_, rho_;
  VectorFiniteVolumeField u_;
  FiniteVolumeEquation<Scalar> pEqn_;
};

template <class T> static bool get(FILE *f, T *p, size_t n) {
  return std::fread(p, sizeof(T), n, f) == n;
}

int main(int argc, char **argv) {
  if (argc < 3) return 2;
  FILE *in = std::fopen(argv[1], "rb");
  if (!in) return 3;
  int64_t nn, nc, nf;
  if (!get(in, &nn, 1) || !get(in, &nc, 1) || !get(in, &nf, 1)) return 4;
  std::vector<Scalar> xy(2 * nn);
  std::vector<int64_t> cptr(nc + 1);
  if (!get(in, xy.data(), xy.size()) || !get(in, cptr.data(), cptr.size())) return 4;
  std::vector<int64_t> cind(cptr[nc]);
  std::vector<Scalar> rho_c(nc), rho_f(nf), uf(2 * nf), pf(nf);
  std::vector<int32_t> bc(nf);
  Scalar dt, tol;
  if (!get(in, cind.data(), cind.size()) || !get(in, rho_c.data(), nc) ||
      !get(in, rho_f.data(), nf) || !get(in, uf.data(), 2 * nf) ||
      !get(in, bc.data(), nf) || !get(in, pf.data(), nf) || !get(in, &dt, 1) ||
      !get(in, &tol, 1))
    return 4;
  std::fclose(in);

  auto grid = std::make_shared<const FiniteVolumeGrid2D>(xy, cptr, cind);
  if ((int64_t)grid->faces().size() != nf) return 5;
  MultiphasePressureStep step(grid);
  for (int64_t c = 0; c < nc; ++c) step.rho_[c] = rho_c[c];
  for (const Face &face : grid->faces()) {
    const Label f = face.id();
    step.rho_(face) = rho_f[f];
    step.u_(face) = Vector2D(uf[2 * f], uf[2 * f + 1]);
    step.p_(face) = pf[f];
    if (face.isBoundary())
      step.p_.setBoundaryType(face, bc[f] == 0 ? ScalarFiniteVolumeField::FIXED
                                               : ScalarFiniteVolumeField::NORMAL_GRADIENT);
  }
  boost::property_tree::ptree keys;
  char tol_s[32];
  std::snprintf(tol_s, sizeof tol_s, "%.17g", tol);
  keys.put("tolerance", tol_s);
  keys.put("maxIters", "20000");
  step.pEqn_.configureSparseSolver(keys);

  const Scalar error = step.solvePEqn(dt);

  FILE *out = std::fopen(argv[2], "wb");
  if (!out) return 6;
  const int32_t iters = step.pEqn_.nIters();
  std::fwrite(step.p_.data(), sizeof(Scalar), nc, out);
  std::fwrite(&error, sizeof(Scalar), 1, out);
  std::fwrite(&iters, sizeof(int32_t), 1, out);
  std::fclose(out);
  std::printf("solvePEqn: %d iterations, error %.3e\n", iters, error);
  return error <= tol ? 0 : 1;
}
