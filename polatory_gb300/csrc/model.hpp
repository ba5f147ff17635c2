// Host-side model description (Model<3>, include/polatory/model.hpp:23-183) and helpers.
#pragma once

#include <cmath>
#include <string>
#include <vector>

#include "common.hpp"
#include "rbf.cuh"

namespace pgpu {

struct RbfDesc {
  int kind = PGPU_RBF_BH3;
  double p[2] = {1.0, 0.0};
  double a[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};

  bool aniso_is_identity() const {
    static const double id[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    for (int i = 0; i < 9; ++i)
      if (a[i] != id[i]) return false;
    return true;
  }
  int cpd_order() const { return kind_cpd_order(kind); }
};

// basis_size (polynomial/polynomial_basis_base.hpp:26-45), 3-D.
inline int poly_basis_size(int degree) {
  if (degree < 0) return 0;
  int k = degree + 1;
  return k * (k + 1) * (k + 2) / 6;
}

struct ModelDesc {
  std::vector<RbfDesc> rbfs;
  int poly_degree = -1;
  double nugget = 0.0;

  int l() const { return poly_basis_size(poly_degree); }
  int cpd_order() const {
    int o = 0;
    for (const auto& r : rbfs) o = std::max(o, r.cpd_order());
    return o;
  }
};

inline double det3(const double* a) {
  return a[0] * (a[4] * a[8] - a[5] * a[7]) - a[1] * (a[3] * a[8] - a[5] * a[6]) +
         a[2] * (a[3] * a[7] - a[4] * a[6]);
}

// Validates and converts the C description: the same checks as model.hpp:32-50 (poly degree
// range), model.hpp:135-141 (nugget) and rbf_base.hpp:70-76 (anisotropy determinant).
inline ModelDesc model_from_c(const pgpu_model* m) {
  if (m == nullptr) throw_invalid("model must not be null");
  if (m->n_rbfs < 1) throw_invalid("rbfs must not be empty");
  if (m->n_rbfs > PGPU_MAX_RBFS) throw_invalid("too many rbfs");
  ModelDesc d;
  for (int i = 0; i < m->n_rbfs; ++i) {
    const pgpu_rbf& r = m->rbfs[i];
    if (r.kind < 0 || r.kind >= PGPU_RBF_COUNT) throw_invalid("unknown RBF kind");
    if (!(det3(r.aniso) > 0.0)) throw_invalid("aniso must have a positive determinant");
    RbfDesc rd;
    rd.kind = r.kind;
    rd.p[0] = r.params[0];
    rd.p[1] = r.params[1];
    for (int k = 0; k < 9; ++k) rd.a[k] = r.aniso[k];
    d.rbfs.push_back(rd);
  }
  int min_deg = d.cpd_order() - 1;
  int deg = m->poly_degree;
  if (deg == -2) deg = min_deg;  // kMinRequiredPolyDegree (model.hpp:28-30)
  if (deg < min_deg || deg > 2) {
    throw_invalid("poly_degree must be within " + std::to_string(min_deg) + " to 2");
  }
  d.poly_degree = deg;
  if (!(m->nugget >= 0.0)) throw_invalid("nugget must be non-negative");
  d.nugget = m->nugget;
  return d;
}

}  // namespace pgpu
