// Fit / evaluate orchestration on the device.
//
// Plain path (PGPU_PRECISION_PLAIN): the reference's Solver::solve loop (interpolation/
// solver.hpp:76-142): FGMRES with the RAS right preconditioner on the FP64 operator; every
// iteration forms the solution vector and checks the absolute inf-norm residual first at up to
// 1024 sampled data points (exact direct sums), then at all points.
//
// Mixed path (PGPU_PRECISION_MIXED): iterative refinement. The outer loop recomputes the
// residual with the FP64 operator (same convergence test as above); each inner FGMRES runs the
// FP32 operator and an FP32 RAS preconditioner with FP64 Krylov vectors, Arnoldi and Givens.
// Mixed precision engages FP32 sums only where they pay: fits and evaluations of at most
// kMixedMinPairs source-target pairs keep FP64 sums (they are cheap, and small systems with
// cancelling weights need FP64 sums to reach 1e-5-level tolerances); such fits still factor
// and apply the preconditioner in FP32, the part of a small fit that costs the most, unless
// the kernel's conditional positive definiteness order is 2 or more.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <functional>
#include <numeric>
#include <random>

#include "linalg.hpp"
#include "ras.hpp"
#include "solver.hpp"

namespace pgpu {

namespace {

// Raised by the mixed path when an FP32 stage produced a non-finite value; fit() then runs the
// plain FP64 path instead.
struct NonFinite : Error {
  NonFinite() : Error(PGPU_RUNTIME_ERROR, "non-finite value in the mixed-precision solve") {}
};

// 2^30 pairs: an FP64 direct sum of this size takes a few milliseconds.
constexpr double kMixedMinPairs = 1073741824.0;

bool mixed_pays(double sources, double targets) { return sources * targets > kMixedMinPairs; }

// y = (A + nugget I) w + P c ; y_tail = P^T w   (interpolation/operator.hpp:56-82).
template <class T>
class Operator {
 public:
  // With sigma gradient points the rows are the mu values then 3 sigma derivatives, and P
  // has mu + 3 sigma rows.
  Operator(const ModelDesc& model, const double* pts_dev, Index mu, const Bbox3& bbox,
           double accuracy, const double* P, const double* grad_dev = nullptr, Index sigma = 0)
      : model_(model), mu_(mu), rows_(mu + 3 * sigma), l_(model.l()),
        ev_(model, bbox, accuracy, accuracy), P_(P) {
    ev_.set_points(pts_dev, mu, grad_dev, sigma);
  }
  Index size() const { return rows_ + l_; }
  // Far-field interpolation order of the operator's FMM (0: from the accuracy).
  void set_order(int p) {
    FarFieldConfig c;
    c.order = p;
    ev_.set_far_field(c);
  }
  void apply(const double* w, double* y) {
    ev_.set_weights(w);
    ev_.evaluate(y, false);
    if (model_.nugget != 0.0) axpy(mu_, model_.nugget, w, y);
    if (l_ > 0) {
      std::vector<double> c(l_), pt(l_);
      PGPU_CUDA(cudaMemcpyAsync(c.data(), w + rows_, l_ * sizeof(double), cudaMemcpyDeviceToHost,
                                stream()));
      sync();
      tall_gemv_add(P_, rows_, l_, c.data(), y);
      tall_gemv_t(P_, rows_, l_, w, pt.data());
      PGPU_CUDA(cudaMemcpyAsync(y + rows_, pt.data(), l_ * sizeof(double), cudaMemcpyHostToDevice,
                                stream()));
      sync();
    }
  }
  Evaluator<T>& evaluator() { return ev_; }

 private:
  const ModelDesc& model_;
  Index mu_;
  Index rows_;
  int l_;
  Evaluator<T> ev_;
  const double* P_;
};

// FGMRES with device-resident V and Z bases; R, Givens rotations and g on the host
// (src/krylov/gmres_base.cpp, gmres.cpp, fgmres.cpp).
class Fgmres {
 public:
  Fgmres(Index m, int max_iter) : m_(m), max_iter_(max_iter) {
    V_.resize(static_cast<size_t>(max_iter + 1) * m);
    Z_.resize(static_cast<size_t>(std::max(max_iter, 1)) * m);
    x0_.resize(m);
    r_.assign(static_cast<size_t>(max_iter + 1) * std::max(max_iter, 1), 0.0);
    c_.assign(std::max(max_iter, 1), 0.0);
    s_.assign(std::max(max_iter, 1), 0.0);
    g_.assign(max_iter + 1, 0.0);
  }

  template <class Op>
  void setup(const double* rhs, const double* x0, bool x0_zero, Op& op) {
    double* v0 = V_.data();
    if (x0_zero) {
      x0_.zero();
      copy(v0, rhs, m_);
    } else {
      copy(x0_.data(), x0, m_);
      op.apply(x0_.data(), v0);
      axpby(m_, 1.0, rhs, -1.0, v0);
    }
    rhs_norm_ = norm2(rhs, m_);
    g_[0] = norm2(v0, m_);
    if (g_[0] > 0) scal(m_, 1.0 / g_[0], v0);
    iter_ = 0;
  }

  template <class Op, class Pc>
  void iterate(Op& op, Pc& pc) {
    if (iter_ == max_iter_) return;
    const int j = iter_;
    double* vj = V_.data() + static_cast<Index>(j) * m_;
    double* z = Z_.data() + static_cast<Index>(j) * m_;
    double* w = V_.data() + static_cast<Index>(j + 1) * m_;
    pc.apply(vj, z);
    op.apply(z, w);
    // Classical Gram-Schmidt: all dots first, then one fused subtraction + norm.
    std::vector<double> h(j + 1);
    multi_dot(V_.data(), m_, j + 1, w, m_, h.data());
    double nrm2 = multi_axpy_sub_norm2(V_.data(), m_, j + 1, h.data(), w, m_);
    double hn = std::sqrt(nrm2);
    for (int i = 0; i <= j; ++i) R(i, j) = h[i];
    R(j + 1, j) = hn;
    if (hn > 0) scal(m_, 1.0 / hn, w);
    for (int i = 0; i < j; ++i) {
      double x = R(i, j), y = R(i + 1, j);
      R(i, j) = c_[i] * x + s_[i] * y;
      R(i + 1, j) = -s_[i] * x + c_[i] * y;
    }
    double x = R(j, j), y = R(j + 1, j);
    double den = std::hypot(x, y);
    c_[j] = x / den;
    s_[j] = y / den;
    R(j, j) = c_[j] * x + s_[j] * y;
    g_[j + 1] = -s_[j] * g_[j];
    g_[j] = c_[j] * g_[j];
    ++iter_;
  }

  // x = x0 + sum_i y_i z_i with R y = g (fgmres.cpp:8-26).
  void solution(double* x) {
    std::vector<double> y(iter_, 0.0);
    for (int j = iter_ - 1; j >= 0; --j) {
      double v = g_[j];
      for (int i = j + 1; i < iter_; ++i) v -= R(j, i) * y[i];
      y[j] = v / R(j, j);
    }
    copy(x, x0_.data(), m_);
    multi_axpy(Z_.data(), m_, iter_, y.data(), x, m_);
  }

  int iteration_count() const { return iter_; }
  int max_iterations() const { return max_iter_; }
  double absolute_residual() const { return std::fabs(g_[iter_]); }
  double relative_residual() const { return std::fabs(g_[iter_]) / rhs_norm_; }

 private:
  double& R(int i, int j) { return r_[static_cast<size_t>(i) * std::max(max_iter_, 1) + j]; }

  Index m_;
  int max_iter_;
  int iter_ = 0;
  double rhs_norm_ = 0;
  DevBuf<double> V_, Z_, x0_;
  std::vector<double> r_, c_, s_, g_;
};

struct Convergence {
  bool converged = false;
  double residual = 0;
  double grad_residual = 0;
  bool exact = false;
  double probe_rms = 0;  // root mean square of the exact residual at the probe points
};

// ResidualEvaluator (residual_evaluator.hpp:56-151). With gradient points the values hold
// mu values then 3 sigma derivatives, and the gradient residual is checked against its own
// tolerance.
class ResidualEvaluator {
 public:
  static constexpr Index kDirectTargets = 1024;

  ResidualEvaluator(const ModelDesc& model, const double* pts_dev, const double* pts_host, Index mu,
                    const Bbox3& bbox, double accuracy, const double* values_host, int precision,
                    const double* grad_dev = nullptr, const double* grad_host = nullptr,
                    Index sigma = 0, double grad_accuracy = INFINITY)
      : model_(model), mu_(mu), sigma_(sigma), l_(model.l()), pts_dev_(pts_dev),
        grad_dev_(grad_dev), bbox_(bbox), accuracy_(accuracy), grad_accuracy_(grad_accuracy),
        precision_(precision) {
    // Probe points: std::shuffle with a default-seeded std::mt19937, then the non-zero values
    // first (residual_evaluator.hpp:119-124); the gradient points the same way with a fresh
    // generator, non-zero gradients first (:126-132).
    std::vector<Index> idx(mu_);
    std::iota(idx.begin(), idx.end(), Index{0});
    std::shuffle(idx.begin(), idx.end(), std::mt19937{});
    std::partition(idx.begin(), idx.end(), [&](Index i) { return values_host[i] != 0.0; });
    n_probe_ = std::min(mu_, kDirectTargets);
    idx.resize(n_probe_);
    probe_idx_.upload(idx);
    std::vector<Index> gidx(sigma_);
    std::iota(gidx.begin(), gidx.end(), Index{0});
    std::shuffle(gidx.begin(), gidx.end(), std::mt19937{});
    std::partition(gidx.begin(), gidx.end(), [&](Index j) {
      const double* g = values_host + mu_ + 3 * j;
      return g[0] != 0.0 || g[1] != 0.0 || g[2] != 0.0;
    });
    n_gprobe_ = std::min(sigma_, kDirectTargets);
    gidx.resize(n_gprobe_);
    std::vector<double> pp(3 * n_probe_), pv(n_probe_ + 3 * n_gprobe_), gp(3 * n_gprobe_);
    for (Index i = 0; i < n_probe_; ++i) {
      for (int k = 0; k < 3; ++k) pp[3 * i + k] = pts_host[3 * idx[i] + k];
      pv[i] = values_host[idx[i]];
    }
    for (Index j = 0; j < n_gprobe_; ++j)
      for (int k = 0; k < 3; ++k) {
        gp[3 * j + k] = grad_host[3 * gidx[j] + k];
        pv[n_probe_ + 3 * j + k] = values_host[mu_ + 3 * gidx[j] + k];
      }
    probe_pts_.upload(pp);
    probe_grad_pts_.upload(gp);
    probe_values_.upload(pv);
    values_.upload(values_host, mu_ + 3 * sigma_);
    fit_.resize(std::max<Index>(mu_ + 3 * sigma_, 1));
    tmp_.resize(std::max<Index>(n_probe_, 1));
  }

  // values - fit at the probe points with exact FP64 sums (device, n_probe()).
  const double* probe_residual(const double* w) {
    probe64().set_weights(w);
    probe64().evaluate(fit_.data());
    if (model_.nugget != 0.0) {
      gather(w, probe_idx_.data(), n_probe_, tmp_.data());
      axpy(n_probe_, model_.nugget, tmp_.data(), fit_.data());
    }
    axpby(n_probe_, 1.0, probe_values_.data(), -1.0, fit_.data());
    return fit_.data();
  }
  // Far-field order of the full check when no accuracy was requested (the reference's default,
  // order 6, resolves residuals down to about 1e-5 of the data scale).
  void set_default_order(int p) {
    if (std::isfinite(accuracy_) && accuracy_ > 0.0) return;
    order_ = p;
    if (full_) {
      FarFieldConfig c;
      c.order = p;
      full_->set_far_field(c);
    }
  }
  Index n_probe() const { return n_probe_; }
  const Index* probe_idx() const { return probe_idx_.data(); }

  Convergence converged(const double* w, double tol, double grad_tol = INFINITY) {
    Convergence cv;
    const double nugget = model_.nugget;
    // Stage 1: exact FP64 sums at the probe points (both precisions: the convergence test is
    // never taken in reduced precision).
    {
      probe64().set_weights(w);
      probe64().evaluate(fit_.data());
      if (nugget != 0.0) {
        gather(w, probe_idx_.data(), n_probe_, tmp_.data());
        axpy(n_probe_, nugget, tmp_.data(), fit_.data());
      }
      cv.residual = inf_norm_diff(fit_.data(), probe_values_.data(), n_probe_);
      cv.grad_residual = inf_norm_diff(fit_.data() + n_probe_, probe_values_.data() + n_probe_,
                                       3 * n_gprobe_);
      const Index np_all = n_probe_ + 3 * n_gprobe_;
      axpby(np_all, 1.0, probe_values_.data(), -1.0, fit_.data());
      cv.probe_rms = norm2(fit_.data(), np_all) / std::sqrt(static_cast<double>(std::max<Index>(np_all, 1)));
      cv.exact = n_probe_ == mu_ && n_gprobe_ == sigma_;
      if (cv.residual > tol || cv.grad_residual > grad_tol) return cv;
      if (cv.exact) {
        cv.converged = true;
        return cv;
      }
    }
    // Stage 2: all points at the requested accuracy.
    full().set_weights(w);
    full().evaluate(fit_.data());
    if (nugget != 0.0) axpy(mu_, nugget, w, fit_.data());
    cv.residual = inf_norm_diff(fit_.data(), values_.data(), mu_);
    cv.grad_residual = inf_norm_diff(fit_.data() + mu_, values_.data() + mu_, 3 * sigma_);
    cv.exact = true;
    cv.converged = cv.residual <= tol && cv.grad_residual <= grad_tol;
    return cv;
  }

 private:
  Evaluator<double>& probe64() {
    if (!p64_) {
      p64_ = std::make_unique<Evaluator<double>>(model_, bbox_, INFINITY, INFINITY);
      p64_->force_direct(true);
      p64_->set_ff_direct(precision_ == PGPU_PRECISION_MIXED);
      p64_->set_sources(pts_dev_, mu_, grad_dev_, sigma_);
      p64_->set_targets(probe_pts_.data(), n_probe_, probe_grad_pts_.data(), n_gprobe_);
    }
    return *p64_;
  }
  Evaluator<float>& probe32() {
    if (!p32_) {
      p32_ = std::make_unique<Evaluator<float>>(model_, bbox_, INFINITY, INFINITY);
      p32_->force_direct(true);
      p32_->set_sources(pts_dev_, mu_, nullptr, 0);
      p32_->set_targets(probe_pts_.data(), n_probe_, nullptr, 0);
    }
    return *p32_;
  }
  Evaluator<double>& full() {
    if (!full_) {
      full_ = std::make_unique<Evaluator<double>>(model_, bbox_, accuracy_, grad_accuracy_);
      full_->set_ff_direct(precision_ == PGPU_PRECISION_MIXED);
      if (order_ > 0) {
        FarFieldConfig c;
        c.order = order_;
        full_->set_far_field(c);
      }
      full_->set_points(pts_dev_, mu_, grad_dev_, sigma_);
    }
    return *full_;
  }

  const ModelDesc& model_;
  Index mu_;
  Index sigma_;
  int l_;
  const double* pts_dev_;
  const double* grad_dev_;
  Bbox3 bbox_;
  double accuracy_;
  double grad_accuracy_;
  int precision_;
  int order_ = 0;
  Index n_probe_ = 0;
  Index n_gprobe_ = 0;
  DevBuf<Index> probe_idx_;
  DevBuf<double> probe_pts_, probe_grad_pts_, probe_values_, values_, fit_, tmp_;
  std::unique_ptr<Evaluator<double>> p64_;
  std::unique_ptr<Evaluator<float>> p32_;
  std::unique_ptr<Evaluator<double>> full_;
};

// Orthogonalises the RBF part of w against the orthonormalised polynomial basis Q
// (solver.hpp:88-92).
void project_out(const double* Q, Index mu, int l, double* w) {
  if (l == 0) return;
  std::vector<double> d(l);
  tall_gemv_t(Q, mu, l, w, d.data());
  for (auto& v : d) v = -v;
  tall_gemv_add(Q, mu, l, d.data(), w);
}

template <class T>
FitResult fit_impl(const FitRequest& req) {
  FitResult res;
  const ModelDesc& model = *req.model;
  const Index mu = req.mu;
  const Index sigma = req.sigma;
  const Index R = mu + 3 * sigma;  // rows: values, then three derivatives per gradient point
  const int l = model.l();
  const Index M = R + l;
  double t0 = wall_seconds();

  DevBuf<double> pts, gpts;
  pts.upload(req.points_host, 3 * mu);
  if (sigma > 0) gpts.upload(req.grad_points_host, 3 * sigma);
  if (req.verbose) {
    sync();
    std::printf("fit: upload %.3f s\n", wall_seconds() - t0);
  }
  Bbox3 bbox = Bbox3::from_host_points(req.points_host, mu);
  if (sigma > 0) bbox = bbox.hull(Bbox3::from_host_points(req.grad_points_host, sigma));
  if (req.verbose) std::printf("fit: bbox %.3f s\n", wall_seconds() - t0);

  DevBuf<double> P, Q;
  if (l > 0) {
    P.resize(R * l);
    monomial_basis(model.poly_degree, pts.data(), mu, gpts.data(), sigma, P.data());
    Q.resize(R * l);
    copy(Q.data(), P.data(), R * l);
    // Modified Gram-Schmidt (common/orthonormalize.hpp:8-18).
    for (int i = 0; i < l; ++i) {
      double* ci = Q.data() + static_cast<Index>(i) * R;
      scal(R, 1.0 / norm2(ci, R), ci);
      for (int j = i + 1; j < l; ++j) {
        double* cj = Q.data() + static_cast<Index>(j) * R;
        axpy(R, -dot(ci, cj, R), ci, cj);
      }
    }
  }

  if (req.verbose) std::printf("fit: basis %.3f s\n", wall_seconds() - t0);
  RasPreconditioner<T> pc(model, req.points_host, pts.data(), mu, req.grad_points_host,
                          gpts.data(), sigma, bbox);
  res.levels = pc.levels();
  res.n_domains = pc.n_domains();
  if (req.verbose) std::printf("fit: preconditioner ready %.3f s\n", wall_seconds() - t0);

  DevBuf<double> w(M), rhs(M);
  w.zero();
  bool x0_zero = true;
  if (req.initial_weights) {
    w.upload(req.initial_weights, M);
    project_out(Q.data(), R, l, w.data());
    x0_zero = false;
  }
  rhs.zero();
  PGPU_CUDA(cudaMemcpyAsync(rhs.data(), req.values_host, R * sizeof(double),
                            cudaMemcpyHostToDevice, stream()));
  sync();

  ResidualEvaluator re(model, pts.data(), req.points_host, mu, bbox, req.accuracy, req.values_host,
                       req.precision, gpts.data(), req.grad_points_host, sigma, req.grad_accuracy);
  res.setup_seconds = wall_seconds() - t0;
  double t1 = wall_seconds();

  if (req.precision == PGPU_PRECISION_PLAIN || req.plain_loop) {
    // Operator at accuracy 0 as interpolation/solver.hpp:40.
    Operator<double> op(model, pts.data(), mu, bbox, 0.0, P.data(), gpts.data(), sigma);
    // Mixed requests below the FP32 threshold: FP64-class float-float direct sums where they
    // exist (odd polyharmonic kernels).
    op.evaluator().set_ff_direct(req.precision == PGPU_PRECISION_MIXED);
    Fgmres solver(M, req.max_iter);
    solver.setup(rhs.data(), w.data(), x0_zero, op);
    if (!x0_zero && solver.relative_residual() == 0.0) {
      res.weights = w.to_host();
      return res;
    }
    if (req.verbose) std::printf("%8s%16s\n", "iter", "residual");
    // The reference's operator (accuracy 0) interpolates the far field at a high order. Here the
    // operator starts at order 6; when the Krylov residual estimate (root mean square) has run
    // ten times below the exact residual's root mean square at the probe points while the check
    // fails, the operator's far-field error is what remains: the order of the operator (and of
    // the full residual check, unless an accuracy was given) is raised to 8 once, FGMRES
    // restarting from the current weights.
    // Gradient data starts at order 8: the derivative blocks lose accuracy against the values at
    // the same order. After order 8 the last rung is exact sums (up to 2^42 pairs), where the
    // reference interpolates at order 12.
    int order = sigma > 0 ? 8 : 6;
    op.set_order(order);
    if (order == 8) re.set_default_order(8);
    const bool exact_ok = static_cast<double>(R) * static_cast<double>(R) <= 4398046511104.0;
    int base = 0;
    while (true) {
      solver.solution(w.data());
      Convergence cv = re.converged(w.data(), req.tolerance, req.grad_tolerance);
      const int total = base + solver.iteration_count();
      if (req.verbose) {
        if (sigma > 0)
          std::printf("%8d%4s%12.6e%4s%12.6e\n", total, cv.exact ? "" : "~", cv.residual,
                      cv.exact ? "" : "~", cv.grad_residual);
        else
          std::printf("%8d%4s%12.6e\n", total, cv.exact ? "" : "~", cv.residual);
      }
      res.residual = cv.residual;
      res.grad_residual = cv.grad_residual;
      if (sizeof(T) == 4 && !std::isfinite(solver.absolute_residual())) throw NonFinite();
      if (cv.converged) break;
      if (total >= req.max_iter)
        throw Error(PGPU_MAX_ITER, "reached the maximum number of iterations");
      const double est_rms = solver.absolute_residual() / std::sqrt(static_cast<double>(R));
      if ((order < 8 || (order == 8 && exact_ok)) && solver.iteration_count() > 0 &&
          est_rms < 0.1 * cv.probe_rms) {
        if (order < 8) {
          order = 8;
          op.set_order(order);
          re.set_default_order(order);
          if (req.verbose) std::printf("%8d    operator order %d\n", total, order);
        } else {
          order = 9;  // exact sums
          op.evaluator().force_direct(true);
          if (req.verbose) std::printf("%8d    operator: exact sums\n", total);
        }
        base = total;
        solver.setup(rhs.data(), w.data(), false, op);
        continue;
      }
      if (solver.iteration_count() == solver.max_iterations()) {
        base = total;
        solver.setup(rhs.data(), w.data(), false, op);
      }
      solver.iterate(op, pc);
    }
    res.iterations = base + solver.iteration_count();
  } else {
    // Iterative refinement: FP64 residuals, FP32 inner solves. Only systems above
    // kMixedMinPairs reach this path.
    // Operators on one FP32 tree, in three grades: FP32 (near field with leaf-relative FP32
    // coordinates and FP64 accumulation of every tile), hybrid (FP64 near field, FP32 far
    // field: the FP32 terms' rounding of large cancelling weights lives in the near field) and
    // the FP64 operator.
    // Residuals are taken with the hybrid operator. One it finds within the tolerance is
    // accepted as the reference accepts its FMM residual (residual_evaluator.hpp:93-107), with
    // exact FP64 sums at up to 1024 sampled data points (the probe points of
    // residual_evaluator.hpp:119-124) within the tolerance too, and one more condition: the
    // residual operator's largest deviation from the exact one at the probes is at most half
    // the tolerance (the check resolves the tolerance). Otherwise residuals are taken with the
    // next grade from then on.
    Operator<float> op32(model, pts.data(), mu, bbox, 0.0, P.data());
    op32.set_order(6);  // the tensor-core M2L's order; refinement absorbs its truncation
    std::unique_ptr<Operator<double>> op64;
    auto fp64_op = [&] {
      if (!op64) {
        op64 = std::make_unique<Operator<double>>(model, pts.data(), mu, bbox, 0.0, P.data());
        op64->set_order(8);
      }
      return op64.get();
    };
    // Grades: FP32 (order 6); hybrid (FP64-class near field, FP32 far field at order 6);
    // hybrid at order 8 (for kernels whose far field order 6 does not resolve the tolerance,
    // such as short-range covariances at coarse levels); FP64 at order 8.
    enum Grade { kFp32 = 0, kHybrid = 1, kHybrid8 = 2, kFp64 = 3 };
    std::unique_ptr<Operator<float>> op32_8;
    auto apply_graded = [&](int grade, const double* x, double* y) {
      if (grade == kFp64) {
        fp64_op()->apply(x, y);
        return;
      }
      Operator<float>* op = &op32;
      if (grade == kHybrid8) {
        if (!op32_8) {
          op32_8 = std::make_unique<Operator<float>>(model, pts.data(), mu, bbox, 0.0, P.data());
          op32_8->set_order(8);
        }
        op = op32_8.get();
      }
      op->evaluator().set_near_fp64(grade != kFp32);
      op->apply(x, y);
      op->evaluator().set_near_fp64(false);
    };
    int residual_grade = kHybrid;
    DevBuf<double> r(M), zero(M), rp32(std::max<Index>(re.n_probe(), 1));
    zero.zero();
    auto residual = [&] {  // r = rhs - A w; returns the inf-norm over the data points
      apply_graded(residual_grade, w.data(), r.data());
      axpby(M, 1.0, rhs.data(), -1.0, r.data());
      return inf_norm_diff(r.data(), zero.data(), mu);
    };
    // One FGMRES with the FP32 preconditioner. Its residual estimate |g_j| (a 2-norm) gives a
    // free necessary condition: while |g_j| / sqrt(mu) exceeds the tolerance the inf-norm does
    // too. Once it passes, the true residual is recomputed at every data point (the absolute
    // inf-norm test of residual_evaluator.hpp:93-107). When the estimate has run far below the
    // true residual (the inner operator's rounding floor), FGMRES restarts from the current
    // weights on the recomputed residual: iterative refinement.
    // Inner operator: FP32; each restart cycle that fails to halve the recomputed residual (the
    // system is too ill-conditioned for this grade at this tolerance) moves it one grade up.
    struct InnerOp {
      Operator<float>* f32;
      std::function<void(int, const double*, double*)> apply_at;
      int grade = 0;
      Index size() const { return f32->size(); }
      void apply(const double* x, double* y) { apply_at(grade, x, y); }
    } inner{&op32, apply_graded};
    int total = 0;
    Fgmres solver(M, req.max_iter);
    // Iterative refinement: w = wb + the current cycle's FGMRES solution. The first cycle solves
    // for the data from the initial weights (wb = 0); every later cycle solves
    // A_inner d = r from zero for the recomputed residual r = rhs - A w, and wb holds the
    // weights it started from.
    DevBuf<double> wb(M), dw(M);
    wb.zero();
    solver.setup(rhs.data(), w.data(), x0_zero, inner);
    auto current = [&] {
      solver.solution(dw.data());
      copy(w.data(), wb.data(), M);
      axpy(M, 1.0, dw.data(), w.data());
    };
    int base = 0;  // iterations before the current cycle
    double cycle_start_residual = INFINITY;
    // Ratio of the inf-norm to the root mean square of the last recomputed residual. The next
    // check waits until the estimate times this ratio predicts at most twice the tolerance.
    double peak_ratio = 1.0;
    // Once residuals need an order-8 or FP64 far field (a check then costs several inner
    // iterations), a refinement cycle is checked only after its estimate has fallen ten times
    // below the residual it started from, and again only after a further fourfold drop.
    double check_below = INFINITY;
    while (true) {
      const double est_rms = solver.absolute_residual() / std::sqrt(static_cast<double>(mu));
      total = base + solver.iteration_count();
      const bool fresh = solver.iteration_count() == 0;
      if (fresh && x0_zero && base == 0) {
        // Zero weights: the residual is the data itself, no operator needed.
        res.residual = inf_norm_diff(rhs.data(), zero.data(), mu);
        peak_ratio = std::max(1.0, res.residual / est_rms);
        if (req.verbose) std::printf("%8d    %12.6e\n", total, res.residual);
        if (res.residual <= req.tolerance) break;
      } else if (!fresh && std::isfinite(est_rms) &&
                 (est_rms > req.tolerance || est_rms * peak_ratio > 2.0 * req.tolerance ||
                  est_rms > check_below)) {
        if (req.verbose) std::printf("%8d   ~%12.6e (estimate)\n", total, est_rms);
      } else {
        current();
        double rinf = residual();
        bool converged = false;
        // Near the tolerance the residual operator must resolve it: its largest deviation from
        // exact FP64 sums at the probe points must be at most half the tolerance, else the next
        // grade takes the residuals from here on.
        while (residual_grade < kFp64 && rinf <= 4.0 * req.tolerance && std::isfinite(rinf)) {
          const Index np = re.n_probe();
          const double* rp = re.probe_residual(w.data());
          gather(r.data(), re.probe_idx(), np, rp32.data());
          const double dev = inf_norm_diff(rp32.data(), rp, np);
          const double rprobe = inf_norm_diff(rp, zero.data(), np);
          if (req.verbose)
            std::printf("%8d    %12.6e (grade %d), probe %12.6e, deviation %9.3e\n", total, rinf,
                        residual_grade, rprobe, dev);
          if (dev <= 0.5 * req.tolerance) {
            converged = rinf <= req.tolerance && rprobe <= req.tolerance;
            if (converged) rinf = std::max(rinf, rprobe);
            break;
          }
          ++residual_grade;
          cycle_start_residual = INFINITY;  // residuals of another operator
          rinf = residual();
        }
        const double rtrue = norm2(r.data(), M);
        if (!std::isfinite(rinf) || !std::isfinite(rtrue) || !std::isfinite(est_rms))
          throw NonFinite();
        res.residual = rinf;
        if (req.verbose) std::printf("%8d    %12.6e\n", total, rinf);
        if (converged || (residual_grade == kFp64 && rinf <= req.tolerance)) break;
        peak_ratio = std::max(1.0, rinf / (rtrue / std::sqrt(static_cast<double>(M))));
        if (solver.iteration_count() > 0 && solver.absolute_residual() < 0.1 * rtrue) {
          if (rinf > 0.5 * cycle_start_residual) {
            // The last cycle did not halve the residual. If the residual operator's own error
            // is a quarter of the residual or more, it is the residual grade that rises (the
            // refinement was chasing its rounding); otherwise the inner operator's.
            bool raised = false;
            if (residual_grade < kFp64) {
              const Index np = re.n_probe();
              const double* rp = re.probe_residual(w.data());
              gather(r.data(), re.probe_idx(), np, rp32.data());
              const double dev = inf_norm_diff(rp32.data(), rp, np);
              if (dev > 0.25 * rinf) {
                ++residual_grade;
                rinf = residual();
                raised = true;
                if (req.verbose)
                  std::printf("%8d    residual grade %d: %12.6e\n", total, residual_grade, rinf);
                if (rinf <= req.tolerance) {
                  res.residual = rinf;
                  break;
                }
              }
            }
            if (!raised && inner.grade < kFp64) {
              ++inner.grade;
              if (req.verbose)
                std::printf("%8d    inner operator grade %d\n", total, inner.grade);
            }
            cycle_start_residual = raised ? INFINITY : rinf;
          } else {
            cycle_start_residual = rinf;
          }
          // New cycle: A_inner d = r from zero, on top of the current weights.
          base = total;
          copy(wb.data(), w.data(), M);
          solver.setup(r.data(), nullptr, true, inner);
          check_below = residual_grade >= kHybrid8
                            ? 0.1 * solver.absolute_residual() / std::sqrt(static_cast<double>(mu))
                            : INFINITY;
        } else {
          if (!std::isfinite(cycle_start_residual)) cycle_start_residual = rinf;
          // The same cycle goes on: its next check waits for a fourfold drop of the estimate.
          check_below = residual_grade >= kHybrid8 ? 0.25 * est_rms : INFINITY;
        }
      }
      if (total >= req.max_iter)
        throw Error(PGPU_MAX_ITER, "reached the maximum number of iterations");
      solver.iterate(inner, pc);
    }
    current();
    res.iterations = total;
  }
  res.solve_seconds = wall_seconds() - t1;
  res.weights = w.to_host();
  return res;
}

template <class T>
void evaluate_impl(const EvaluateRequest& req) {
  Evaluator<T> ev(*req.model, req.bbox, req.accuracy, req.grad_accuracy);
  ev.set_ff_direct(req.precision == PGPU_PRECISION_MIXED);
  ev.set_sources(req.centers_dev, req.mu, req.grad_centers_dev, req.sigma);
  ev.set_targets(req.points_dev, req.m, req.grad_points_dev, req.mg);
  ev.set_weights(req.weights_dev);
  ev.evaluate(req.out_dev);
}

}  // namespace

namespace {
// Inputs must be finite: a NaN or infinite coordinate would poison the bounding box, the octree
// keys and the domain division (the reference does not check; here they are rejected).
void check_finite_host(const double* p, Index n, const char* what) {
  for (Index i = 0; i < n; ++i)
    if (!std::isfinite(p[i])) throw_invalid(std::string(what) + " must be finite");
}
}  // namespace

FitResult fit(const FitRequest& req) {
  check_finite_host(req.points_host, 3 * req.mu, "points");
  if (req.sigma > 0) {
    check_finite_host(req.grad_points_host, 3 * req.sigma, "grad_points");
    // The gradient-gradient blocks need the kernel's Hessian (mat_a.hpp:44-58).
    for (const auto& rb : req.model->rbfs)
      if (!kind_has_hessian(rb.kind))
        throw_runtime(std::string(rb.kind == PGPU_RBF_CUB ? "cov_cubic" : "cov_spherical") +
                      "::evaluate_hessian_isotropic is not implemented");
  }
  check_finite_host(req.values_host, req.mu + 3 * req.sigma, "values");
  const double mu = static_cast<double>(req.mu);
  FitRequest plain = req;
  plain.precision = PGPU_PRECISION_PLAIN;
  if (req.precision == PGPU_PRECISION_PLAIN) return fit_impl<double>(plain);
  if (req.sigma > 0) {
    // Gradient data: the value/gradient/Hessian blocks run in FP64 (the reference's arithmetic)
    // whatever the requested precision; the result says so.
    return fit_impl<double>(plain);
  }
  auto mixed = [](FitResult r) {
    r.precision_used = PGPU_PRECISION_MIXED;
    return r;
  };
  // Kernels of conditional positive definiteness order 2 and above (triharmonic, thin-plate)
  // give domain matrices too ill-conditioned for an FP32 Cholesky factor: their small fits keep
  // the FP64 preconditioner.
  FitRequest small = req;
  small.plain_loop = true;
  if (!mixed_pays(mu, mu) && req.model->cpd_order() >= 2) return mixed(fit_impl<double>(small));
  try {
    if (!mixed_pays(mu, mu)) {
      // Small systems: FP64-class operator and residuals (direct sums), FP32 preconditioner.
      return mixed(fit_impl<float>(small));
    }
    return mixed(fit_impl<float>(req));
  } catch (const NonFinite&) {
    if (req.verbose) std::printf("fit: non-finite value in FP32, running the FP64 path\n");
    FitResult r = fit_impl<double>(plain);
    r.fell_back = true;
    return r;
  }
}

void evaluate(const EvaluateRequest& req) {
  if (!device_all_finite(req.points_dev, 3 * req.m) ||
      !device_all_finite(req.grad_points_dev, 3 * req.mg))
    throw_invalid("points must be finite");
  const double pairs_src = static_cast<double>(req.mu + req.sigma);
  const double pairs_trg = static_cast<double>(req.m + req.mg);
  if (req.precision == PGPU_PRECISION_PLAIN || !mixed_pays(pairs_src, pairs_trg))
    evaluate_impl<double>(req);
  else
    evaluate_impl<float>(req);
}

namespace {
struct DenseOperator {
  const double* a;
  Index n;
  void apply(const double* x, double* y) { dense_gemv(a, n, x, y); }
};
struct IdentityOperator {
  Index n;
  void apply(const double* x, double* y) { copy(y, x, n); }
};
}  // namespace

void krylov_fgmres_dense(Index n, const double* op, const double* pc, const double* rhs,
                         const double* x0, int iters, double* solutions, double* rel_residuals) {
  if (n <= 0 || iters < 0 || iters > n) throw_invalid("need n > 0 and 0 <= iters <= n");
  DevBuf<double> a, p, b, x0d, x(n);
  a.upload(op, static_cast<size_t>(n * n));
  b.upload(rhs, n);
  if (pc) p.upload(pc, static_cast<size_t>(n * n));
  if (x0) x0d.upload(x0, n);
  DenseOperator A{a.data(), n}, P{p.data(), n};
  IdentityOperator I{n};
  Fgmres g(n, iters);
  g.setup(b.data(), x0 ? x0d.data() : nullptr, x0 == nullptr, A);
  for (int k = 0; k < iters; ++k) {
    if (pc)
      g.iterate(A, P);
    else
      g.iterate(A, I);
    g.solution(x.data());
    x.download(solutions + static_cast<Index>(k) * n, n);
    sync();
    rel_residuals[k] = g.relative_residual();
  }
}

}  // namespace pgpu
