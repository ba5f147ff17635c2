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
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <numeric>
#include <random>

#include "linalg.hpp"
#include "ras.hpp"
#include "solver.hpp"

namespace pgpu {

namespace {

// y = (A + nugget I) w + P c ; y_tail = P^T w   (interpolation/operator.hpp:56-82).
template <class T>
class Operator {
 public:
  Operator(const ModelDesc& model, const double* pts_dev, Index mu, const Bbox3& bbox,
           double accuracy, const double* P)
      : model_(model), mu_(mu), l_(model.l()), ev_(model, bbox, accuracy, accuracy), P_(P) {
    ev_.set_points(pts_dev, mu, nullptr, 0);
  }
  Index size() const { return mu_ + l_; }
  void apply(const double* w, double* y) {
    ev_.set_weights(w);
    ev_.evaluate(y, false);
    if (model_.nugget != 0.0) axpy(mu_, model_.nugget, w, y);
    if (l_ > 0) {
      std::vector<double> c(l_), pt(l_);
      PGPU_CUDA(cudaMemcpyAsync(c.data(), w + mu_, l_ * sizeof(double), cudaMemcpyDeviceToHost,
                                stream()));
      sync();
      tall_gemv_add(P_, mu_, l_, c.data(), y);
      tall_gemv_t(P_, mu_, l_, w, pt.data());
      PGPU_CUDA(cudaMemcpyAsync(y + mu_, pt.data(), l_ * sizeof(double), cudaMemcpyHostToDevice,
                                stream()));
      sync();
    }
  }
  Evaluator<T>& evaluator() { return ev_; }

 private:
  const ModelDesc& model_;
  Index mu_;
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
  bool exact = false;
};

// ResidualEvaluator (residual_evaluator.hpp:56-151), value points only.
class ResidualEvaluator {
 public:
  static constexpr Index kDirectTargets = 1024;

  ResidualEvaluator(const ModelDesc& model, const double* pts_dev, const double* pts_host, Index mu,
                    const Bbox3& bbox, double accuracy, const double* values_host, int precision)
      : model_(model), mu_(mu), l_(model.l()), pts_dev_(pts_dev), bbox_(bbox), accuracy_(accuracy),
        precision_(precision) {
    // Probe points: std::shuffle with a default-seeded std::mt19937, then the non-zero values
    // first (residual_evaluator.hpp:119-124).
    std::vector<Index> idx(mu_);
    std::iota(idx.begin(), idx.end(), Index{0});
    std::shuffle(idx.begin(), idx.end(), std::mt19937{});
    std::partition(idx.begin(), idx.end(), [&](Index i) { return values_host[i] != 0.0; });
    n_probe_ = std::min(mu_, kDirectTargets);
    idx.resize(n_probe_);
    probe_idx_.upload(idx);
    std::vector<double> pp(3 * n_probe_), pv(n_probe_);
    for (Index i = 0; i < n_probe_; ++i) {
      for (int k = 0; k < 3; ++k) pp[3 * i + k] = pts_host[3 * idx[i] + k];
      pv[i] = values_host[idx[i]];
    }
    probe_pts_.upload(pp);
    probe_values_.upload(pv);
    values_.upload(values_host, mu_);
    fit_.resize(std::max<Index>(mu_, 1));
    tmp_.resize(std::max<Index>(n_probe_, 1));
  }

  Convergence converged(const double* w, double tol) {
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
      cv.exact = n_probe_ == mu_;
      if (cv.residual > tol) return cv;
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
    cv.exact = true;
    cv.converged = cv.residual <= tol;
    return cv;
  }

 private:
  Evaluator<double>& probe64() {
    if (!p64_) {
      p64_ = std::make_unique<Evaluator<double>>(model_, bbox_, INFINITY, INFINITY);
      p64_->force_direct(true);
      p64_->set_sources(pts_dev_, mu_, nullptr, 0);
      p64_->set_targets(probe_pts_.data(), n_probe_, nullptr, 0);
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
      full_ = std::make_unique<Evaluator<double>>(model_, bbox_, accuracy_, accuracy_);
      full_->set_points(pts_dev_, mu_, nullptr, 0);
    }
    return *full_;
  }

  const ModelDesc& model_;
  Index mu_;
  int l_;
  const double* pts_dev_;
  Bbox3 bbox_;
  double accuracy_;
  int precision_;
  Index n_probe_ = 0;
  DevBuf<Index> probe_idx_;
  DevBuf<double> probe_pts_, probe_values_, values_, fit_, tmp_;
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
  const int l = model.l();
  const Index M = mu + l;
  double t0 = wall_seconds();

  DevBuf<double> pts;
  pts.upload(req.points_host, 3 * mu);
  const Bbox3 bbox = Bbox3::from_host_points(req.points_host, mu);

  DevBuf<double> P, Q;
  if (l > 0) {
    P.resize(mu * l);
    monomial_basis(model.poly_degree, pts.data(), mu, nullptr, 0, P.data());
    Q.resize(mu * l);
    copy(Q.data(), P.data(), mu * l);
    // Modified Gram-Schmidt (common/orthonormalize.hpp:8-18).
    for (int i = 0; i < l; ++i) {
      double* ci = Q.data() + static_cast<Index>(i) * mu;
      scal(mu, 1.0 / norm2(ci, mu), ci);
      for (int j = i + 1; j < l; ++j) {
        double* cj = Q.data() + static_cast<Index>(j) * mu;
        axpy(mu, -dot(ci, cj, mu), ci, cj);
      }
    }
  }

  if (req.verbose) std::printf("fit: basis %.3f s\n", wall_seconds() - t0);
  RasPreconditioner<T> pc(model, req.points_host, pts.data(), mu, bbox);
  res.levels = pc.levels();
  res.n_domains = pc.n_domains();
  if (req.verbose) std::printf("fit: preconditioner ready %.3f s\n", wall_seconds() - t0);

  DevBuf<double> w(M), rhs(M);
  w.zero();
  bool x0_zero = true;
  if (req.initial_weights) {
    w.upload(req.initial_weights, M);
    project_out(Q.data(), mu, l, w.data());
    x0_zero = false;
  }
  rhs.zero();
  PGPU_CUDA(cudaMemcpyAsync(rhs.data(), req.values_host, mu * sizeof(double),
                            cudaMemcpyHostToDevice, stream()));
  sync();

  ResidualEvaluator re(model, pts.data(), req.points_host, mu, bbox, req.accuracy, req.values_host,
                       req.precision);
  res.setup_seconds = wall_seconds() - t0;
  double t1 = wall_seconds();

  if (req.precision == PGPU_PRECISION_PLAIN) {
    // Operator at accuracy 0 as interpolation/solver.hpp:40.
    Operator<double> op(model, pts.data(), mu, bbox, 0.0, P.data());
    Fgmres solver(M, req.max_iter);
    solver.setup(rhs.data(), w.data(), x0_zero, op);
    if (!x0_zero && solver.relative_residual() == 0.0) {
      res.weights = w.to_host();
      return res;
    }
    if (req.verbose) std::printf("%8s%16s\n", "iter", "residual");
    while (true) {
      solver.solution(w.data());
      Convergence cv = re.converged(w.data(), req.tolerance);
      if (req.verbose)
        std::printf("%8d%4s%12.6e\n", solver.iteration_count(), cv.exact ? "" : "~", cv.residual);
      res.residual = cv.residual;
      if (cv.converged) break;
      if (solver.iteration_count() == solver.max_iterations())
        throw Error(PGPU_MAX_ITER, "reached the maximum number of iterations");
      solver.iterate(op, pc);
    }
    res.iterations = solver.iteration_count();
  } else {
    // Iterative refinement: FP64 residuals, FP32 inner solves.
    // Residual operator: exact FP64 sums while they are cheap; beyond that the FP32 FMM whose
    // near field subtracts leaf-relative coordinates (exact to FP32 rounding of leaf-sized
    // offsets) and accumulates every tile in FP64 — the compensated near-field sum.
    const bool fp64_residual = static_cast<double>(mu) * static_cast<double>(mu) <= 1073741824.0;
    std::unique_ptr<Operator<double>> op64;
    if (fp64_residual) op64 = std::make_unique<Operator<double>>(model, pts.data(), mu, bbox, 0.0, P.data());
    Operator<float> op32(model, pts.data(), mu, bbox, 0.0, P.data());
    DevBuf<double> r(M), zero(M);
    zero.zero();
    // One FGMRES on the FP32 operator. Its residual estimate |g_j| (a 2-norm) gives a free
    // necessary condition: while |g_j| / sqrt(mu) exceeds the tolerance the inf-norm does too.
    // Once it passes, the true residual is recomputed at every data point (the absolute
    // inf-norm test of residual_evaluator.hpp:93-107). When the estimate has run far below the
    // true residual (the FP32 operator's rounding floor), FGMRES restarts from the current
    // weights on the recomputed residual: iterative refinement.
    // Inner operator: FP32 until a restart cycle fails to halve the recomputed residual (the
    // system is too ill-conditioned for FP32 sums at this tolerance); then FP64 for the rest.
    struct InnerOp {
      Operator<float>* f32;
      Operator<double>* f64 = nullptr;
      Index size() const { return f32->size(); }
      void apply(const double* x, double* y) {
        if (f64) f64->apply(x, y);
        else f32->apply(x, y);
      }
    } inner{&op32};
    std::unique_ptr<Operator<double>> op64_inner;
    auto residual_op = [&](const double* x, double* y) {
      if (op64) op64->apply(x, y);
      else if (inner.f64) inner.f64->apply(x, y);
      else op32.apply(x, y);
    };
    int total = 0;
    Fgmres solver(M, req.max_iter);
    solver.setup(rhs.data(), w.data(), x0_zero, inner);
    int base = 0;  // iterations before the current restart
    double cycle_start_residual = INFINITY;
    while (true) {
      const double est_rms = solver.absolute_residual() / std::sqrt(static_cast<double>(mu));
      total = base + solver.iteration_count();
      if (solver.iteration_count() > 0 && est_rms > req.tolerance) {
        if (req.verbose) std::printf("%8d   ~%12.6e (estimate)\n", total, est_rms);
      } else {
        solver.solution(w.data());
        residual_op(w.data(), r.data());
        axpby(M, 1.0, rhs.data(), -1.0, r.data());
        const double rinf = inf_norm_diff(r.data(), zero.data(), mu);
        res.residual = rinf;
        if (req.verbose) std::printf("%8d    %12.6e\n", total, rinf);
        if (rinf <= req.tolerance) break;
        const double rtrue = norm2(r.data(), M);
        if (solver.iteration_count() > 0 && solver.absolute_residual() < 0.1 * rtrue) {
          if (!inner.f64 && rinf > 0.5 * cycle_start_residual) {
            op64_inner = std::make_unique<Operator<double>>(model, pts.data(), mu, bbox, 0.0, P.data());
            inner.f64 = op64_inner.get();
            if (req.verbose) std::printf("%8d    switching the inner operator to FP64\n", total);
          }
          cycle_start_residual = rinf;
          base = total;
          solver.setup(rhs.data(), w.data(), false, inner);
        } else if (!std::isfinite(cycle_start_residual)) {
          cycle_start_residual = rinf;
        }
      }
      if (total >= req.max_iter)
        throw Error(PGPU_MAX_ITER, "reached the maximum number of iterations");
      if (solver.iteration_count() == solver.max_iterations()) {
        solver.solution(w.data());
        base = total;
        solver.setup(rhs.data(), w.data(), false, inner);
      }
      solver.iterate(inner, pc);
    }
    res.iterations = total;
  }
  res.solve_seconds = wall_seconds() - t1;
  res.weights = w.to_host();
  return res;
}

template <class T>
void evaluate_impl(const EvaluateRequest& req) {
  Evaluator<T> ev(*req.model, req.bbox, req.accuracy, req.grad_accuracy);
  ev.set_sources(req.centers_dev, req.mu, req.grad_centers_dev, req.sigma);
  ev.set_targets(req.points_dev, req.m, req.grad_points_dev, req.mg);
  ev.set_weights(req.weights_dev);
  ev.evaluate(req.out_dev);
}

}  // namespace

FitResult fit(const FitRequest& req) {
  if (req.sigma > 0) throw Error(PGPU_NOT_IMPLEMENTED, "gradient data points are not supported yet");
  if (req.precision == PGPU_PRECISION_PLAIN) return fit_impl<double>(req);
  return fit_impl<float>(req);
}

void evaluate(const EvaluateRequest& req) {
  if (req.precision == PGPU_PRECISION_PLAIN) evaluate_impl<double>(req);
  else evaluate_impl<float>(req);
}

}  // namespace pgpu
