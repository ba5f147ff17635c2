// Minimal stand-ins for the reference's types that the C++ binding in INTEGRATION.md touches
// (Model<3>, its RBFs, geometry::Points3, VecX), so that the binding compiles and runs against
// the C ABI without the reference's dependencies. Only the members the binding calls exist.
#pragma once

#include <array>
#include <limits>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

namespace polatory {

using Index = long long;

struct VecX {
  std::vector<double> v;
  explicit VecX(Index n = 0) : v(static_cast<size_t>(n)) {}
  double* data() { return v.data(); }
  const double* data() const { return v.data(); }
  Index rows() const { return static_cast<Index>(v.size()); }
  double& operator()(Index i) { return v[static_cast<size_t>(i)]; }
};

namespace geometry {
struct Points3 {  // row-major n x 3, like the reference's Eigen type
  std::vector<double> v;
  Points3(Index n = 0, Index = 3) : v(static_cast<size_t>(3 * n)) {}
  double* data() { return v.data(); }
  const double* data() const { return v.data(); }
  Index rows() const { return static_cast<Index>(v.size() / 3); }
  double& operator()(Index i, Index k) { return v[static_cast<size_t>(3 * i + k)]; }
};
}  // namespace geometry

struct Mat3 {
  std::array<double, 9> a{1, 0, 0, 0, 1, 0, 0, 0, 1};
  double operator()(int r, int c) const { return a[3 * r + c]; }
};

struct Rbf {
  std::string name;
  std::vector<double> params;
  Mat3 aniso;
  const std::string& short_name() const { return name; }
  const std::vector<double>& parameters() const { return params; }
  const Mat3& anisotropy() const { return aniso; }
};

template <int Dim>
struct Model {
  std::vector<Rbf> rbfs_;
  int degree = 1;
  double nugget_ = 0;
  Index num_rbfs() const { return static_cast<Index>(rbfs_.size()); }
  const std::vector<Rbf>& rbfs() const { return rbfs_; }
  int poly_degree() const { return degree; }
  double nugget() const { return nugget_; }
};

}  // namespace polatory
