// Drives the C++ binding of INTEGRATION.md (included from the extracted code block) against the
// library: a 2,000-point biharmonic fit and an evaluation at the data points.
#include <cmath>
#include <cstdio>

#include "gpu_interpolant.hpp"

int main() {
  using namespace polatory;
  const Index n = 2000;
  geometry::Points3 pts(n, 3);
  VecX vals(n);
  unsigned long long s = 99;
  auto uni = [&] {
    s = s * 6364136223846793005ULL + 1442695040888963407ULL;
    return static_cast<double>(s >> 11) / 9007199254740992.0;
  };
  for (Index i = 0; i < n; ++i) {
    for (int k = 0; k < 3; ++k) pts(i, k) = uni();
    vals(i) = std::sin(6.283185307179586 * pts(i, 0)) + pts(i, 2);
  }
  Model<3> model;
  model.rbfs_.push_back(Rbf{"bh3", {1.0, 0.0}, {}});
  try {
    gpu::Interpolant it(model);
    it.fit(pts, vals, 1e-6);
    VecX out = it.evaluate(pts);
    double err = 0;
    for (Index i = 0; i < n; ++i) err = std::fmax(err, std::fabs(out(i) - vals(i)));
    std::printf("max_error %.3e\n", err);
    // The reference's exception mapping: a bad tolerance is std::invalid_argument.
    try {
      it.fit(pts, vals, -1.0);
      return 3;
    } catch (const std::invalid_argument&) {
    }
    return err <= 2e-6 ? 0 : 2;
  } catch (const std::exception& e) {
    std::fprintf(stderr, "error: %s\n", e.what());
    return 1;
  }
}
