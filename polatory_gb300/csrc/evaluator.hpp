// Evaluator<T>: sum over the model's RBFs of the kernel sums from a source set (value points
// with weights, gradient points with 3-vector weights) to a target set (value points, gradient
// points), plus the polynomial part. This is the device form of interpolation::Evaluator
// (include/polatory/interpolation/evaluator.hpp:18-160) and, with sources == targets, of
// interpolation::SymmetricEvaluator (symmetric_evaluator.hpp:19-128). T is the arithmetic of the
// kernel sums (double for the plain path, float for the mixed path); accumulation, weights and
// outputs are double.
#pragma once

#include <memory>
#include <vector>

#include "common.hpp"
#include "kernels.cuh"
#include "model.hpp"

namespace pgpu {

struct Bbox3 {
  double min[3] = {INFINITY, INFINITY, INFINITY};
  double max[3] = {-INFINITY, -INFINITY, -INFINITY};
  bool empty() const { return min[0] > max[0] || min[1] > max[1] || min[2] > max[2]; }
  Bbox3 hull(const Bbox3& o) const {
    Bbox3 r;
    for (int k = 0; k < 3; ++k) {
      r.min[k] = std::min(min[k], o.min[k]);
      r.max[k] = std::max(max[k], o.max[k]);
    }
    return r;
  }
  static Bbox3 from_host_points(const double* p, Index n) {
    Bbox3 b;
    for (Index i = 0; i < n; ++i)
      for (int k = 0; k < 3; ++k) {
        b.min[k] = std::min(b.min[k], p[3 * i + k]);
        b.max[k] = std::max(b.max[k], p[3 * i + k]);
      }
    return b;
  }
};

// Bounding box of device points (x y z rows).
Bbox3 bbox_of_device_points(const double* pts, Index n);
// True when every one of the n device values is finite (one reduction and a sync).
bool device_all_finite(const double* p, Index n);
// out[3 i ..] += A^T g[3 i ..] for n gradients (device).
void frame_gradient_add(const Mat3& a, const double* g, Index n, double* out);
// Lattice node positions (lc_origin + lc) * basis for n device int32 triples (lcs), into pts (n x 3).
void lattice_positions(const double lc_origin[3], const double basis[9], const int32_t* lcs, Index n,
                       double* pts);
// x[i] -= c on the device.
void subtract_scalar(double* x, Index n, double c);

// FMM / direct configuration selected from an accuracy (fmm_accuracy_estimator.hpp:74-121).
struct FarFieldConfig {
  int order = 0;          // interpolation nodes per axis (0: from the accuracy)
  int leaf_level = -1;    // -1: automatic
  // Near field only, for kernels of compact support: leaves at least near_radius wide (in the
  // anisotropy frame), so that the 27 neighbour leaves hold every source within the support.
  bool near_only = false;
  double near_radius = 0.0;
};

struct EvalStats {
  Index near_pairs = 0;   // P2P pairs in the last evaluate (0 for direct backend)
  Index direct_pairs = 0; // pairs evaluated by the direct backend
  int backend = 0;        // 0 direct, 1 fmm
};

class RbfTermBase {
 public:
  virtual ~RbfTermBase() = default;
};

template <class T>
class Evaluator {
 public:
  Evaluator(const ModelDesc& model, const Bbox3& bbox, double accuracy, double grad_accuracy);
  ~Evaluator();

  // Device xyz rows (double). Arrays must stay valid until the next set_* call.
  void set_sources(const double* pts, Index mu, const double* gpts, Index sigma);
  void set_targets(const double* pts, Index m, const double* gpts, Index mg);
  // Symmetric form: sources == targets.
  void set_points(const double* pts, Index mu, const double* gpts, Index sigma);
  // Device weights [mu + 3 sigma + l].
  void set_weights(const double* w);
  // out (device) [m + 3 mg] = kernel sums + polynomial.
  void evaluate(double* out, bool with_poly = true);

  Index n_sources() const { return mu_ + 3 * sigma_; }
  Index n_targets() const { return m_ + 3 * mg_; }
  const EvalStats& stats() const { return stats_; }
  // Backend choice: automatic (by pair count), exact direct sums, or the FMM where supported.
  static constexpr int kBackendAuto = 0, kBackendDirect = 1, kBackendFmm = 2;
  void set_backend(int b) { backend_ = b; }
  void force_direct(bool f) { backend_ = f ? kBackendDirect : kBackendAuto; }
  // Far-field order / leaf level; applies to FMMs already built too (they rebuild).
  void set_far_field(const FarFieldConfig& c);
  // FP32 evaluators of value sources and targets: near field (or all pairs, on the direct
  // backend) in FP64 from the FP64 coordinates and weights; the far field stays FP32.
  void set_near_fp64(bool on) { near64_ = on; }
  // FP64 evaluators: value-to-value direct sums of the odd polyharmonic kernels in float-float
  // arithmetic (FP64-class accuracy on the FP32 pipes). Off by default (the plain path keeps
  // FP64 arithmetic throughout).
  void set_ff_direct(bool on) { ff_direct_ = on; }

 private:
  struct Term;
  // acc_v bounds the value outputs' error, acc_g the gradient outputs' (used when the
  // evaluator has gradient sources or targets).
  int estimate_order(Term& t, double acc_v, double acc_g);

  ModelDesc model_;
  Bbox3 bbox_;
  double accuracy_, grad_accuracy_;
  bool symmetric_ = false;
  int backend_ = kBackendAuto;
  bool ff_set_ = false;
  FarFieldConfig ff_;
  bool near64_ = false;
  bool ff_direct_ = false;
  const double* w_ = nullptr;  // the weights of the last set_weights (device)
  Index mu_ = 0, sigma_ = 0, m_ = 0, mg_ = 0;
  const double* spts_ = nullptr;
  const double* sgpts_ = nullptr;
  const double* tpts_ = nullptr;
  const double* tgpts_ = nullptr;
  std::vector<std::unique_ptr<Term>> terms_;
  std::vector<double> poly_c_;
  EvalStats stats_;
};

}  // namespace pgpu
