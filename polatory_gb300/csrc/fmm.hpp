// Interpolation-based FMM on a uniform-depth octree of Morton-sorted points.
#pragma once

#include "common.hpp"
#include "evaluator.hpp"
#include "kernels.cuh"

namespace pgpu {

template <class T>
class Fmm {
 public:
  // Kernels whose far field interpolates (the smooth ones, and the spheroidal fast parts).
  static bool supported(int kind);
  // Kernels of compact support, evaluated by near-field-only trees (FarFieldConfig::near_only).
  static bool near_only_supported(int kind);
  // box_min / box_width: the cube (anisotropy frame, relative to the frame origin of the
  // positions handed in later).
  Fmm(int kind, const KParams<T>& kp, const Mat3& a, const double box_min[3], double box_width,
      double accuracy);
  ~Fmm();
  void set_config(const FarFieldConfig& c);
  // Positions in the anisotropy frame (FP64, relative to the frame origin). The tree keeps them
  // relative to their leaf centres in T, which keeps FP32 near-field differences exact to FP32
  // rounding of the (small) leaf-relative offsets.
  void set_points(const P4<double>* pos, Index n);
  void set_sources(const P4<double>* pos, Index n);
  void set_targets(const P4<double>* pos, Index n);
  // Targets are gradient targets: evaluate adds, per target, the three components of the
  // gradient in the anisotropy frame (out_v[3 i + k]; the caller maps them back with A^T).
  // Smooth public kinds only.
  void set_gradient_targets(bool on);
  // Sources are gradient sources: their weights are the three frame components per source (gg
  // of evaluate, A g in the caller's order). Smooth public kinds only; the near field stays in T.
  void set_gradient_sources(bool on);
  // FP32 trees: take the near field with FP64 positions (leaf-relative), weights and sums,
  // the far field staying in T. Ignored for FP64 trees.
  void set_near_fp64(bool on, const KParams<double>& kp64);
  // Adds the potentials (value targets) and A^T-mapped gradients (gradient targets). w64: the
  // FP64 value weights (unsorted), read by an FP64 near field.
  void evaluate(const T* vw, const T* gg, const double* w64, double* out_v, double* out_g);
  Index near_pairs() const;

 private:
  struct Impl;
  Impl* impl_;
};

// The process-wide M2L operator cache: bytes and entries held, and its byte limit
// (PGPU_M2L_CACHE_MB at start-up, 8 GiB by default). Setting the limit evicts down to it.
void m2l_cache_stats(int64_t* bytes, int64_t* entries, int64_t* limit);
void m2l_cache_set_limit(int64_t bytes);

}  // namespace pgpu
