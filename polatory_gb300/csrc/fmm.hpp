// Interpolation-based FMM on a uniform-depth octree of Morton-sorted points.
#pragma once

#include "common.hpp"
#include "evaluator.hpp"
#include "kernels.cuh"

namespace pgpu {

template <class T>
class Fmm {
 public:
  static bool supported(int kind);
  // box_min / box_width: the cube (anisotropy frame, relative to the frame origin of the
  // positions handed in later).
  Fmm(int kind, const KParams<T>& kp, const Mat3& a, const double box_min[3], double box_width,
      double accuracy);
  ~Fmm();
  void set_config(const FarFieldConfig& c);
  void set_points(const P4<T>* pos, Index n, const P4<T>* gpos, Index ng);
  void set_sources(const P4<T>* pos, Index n, const P4<T>* gpos, Index ng);
  void set_targets(const P4<T>* pos, Index n, const P4<T>* gpos, Index ng);
  // Adds the potentials (value targets) and A^T-mapped gradients (gradient targets).
  void evaluate(const T* vw, const T* gg, double* out_v, double* out_g);
  Index near_pairs() const;

 private:
  struct Impl;
  Impl* impl_;
};

}  // namespace pgpu
