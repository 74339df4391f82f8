// Driver around the reference's own CrsEquation (compiled from the
// reference sources into oracle/_ref/libref_crs.so) -- TEST INFRASTRUCTURE.
// It replays a sequence of CrsEquation calls and exports the resulting
// arrays, so the tests can pin the oracle's CSR semantics (placeholder
// slots, slot order, duplicate summing, row growth past the reserved slots,
// operator+= dropping zero and placeholder entries) on the real code.
#include <cstdint>
#include <vector>

#include "Math/CrsEquation.h"

namespace {
struct Handle {
  CrsEquation eqn;
};
}  // namespace

extern "C" {

void *ref_crs_create(int64_t n_rows, int64_t nnz_per_row) {
  auto *h = new Handle();
  h->eqn = CrsEquation((Size)n_rows, (Size)nnz_per_row);
  return h;
}

void ref_crs_destroy(void *h) { delete static_cast<Handle *>(h); }

// op 0: addCoeff(row, col, val); op 1: addRhs(row, val)
void ref_crs_apply(void *hp, int64_t n_ops, const int32_t *op,
                   const int32_t *row, const int32_t *col,
                   const double *val) {
  auto &e = static_cast<Handle *>(hp)->eqn;
  for (int64_t k = 0; k < n_ops; ++k) {
    if (op[k] == 0)
      e.addCoeff(row[k], col[k], val[k]);
    else
      e.addRhs(row[k], val[k]);
  }
}

// eqn == src  (CrsEquation::operator==(const Vector&))
void ref_crs_eq_vector(void *hp, int64_t n, const double *v) {
  auto &e = static_cast<Handle *>(hp)->eqn;
  Vector vec((Size)n);
  for (int64_t i = 0; i < n; ++i) vec(i) = v[i];
  e == vec;
}

// a += b  (CrsEquation::operator+=(const CrsEquation&))
void ref_crs_plus(void *a, const void *b) {
  static_cast<Handle *>(a)->eqn += static_cast<const Handle *>(b)->eqn;
}

void ref_crs_sizes(void *hp, int64_t *n, int64_t *n_slots) {
  auto &e = static_cast<Handle *>(hp)->eqn;
  *n = (int64_t)e.rank();
  *n_slots = (int64_t)e.colInd().size();
}

void ref_crs_export(void *hp, int32_t *row_ptr, int32_t *col_ind,
                    double *vals, double *rhs) {
  auto &e = static_cast<Handle *>(hp)->eqn;
  for (size_t i = 0; i < e.rowPtr().size(); ++i) row_ptr[i] = e.rowPtr()[i];
  for (size_t i = 0; i < e.colInd().size(); ++i) {
    col_ind[i] = e.colInd()[i];
    vals[i] = e.vals()[i];
  }
  for (size_t i = 0; i < e.rank(); ++i) rhs[i] = e.b((Index)i);
}
}
