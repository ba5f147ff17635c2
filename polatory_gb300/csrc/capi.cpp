// The C ABI (include/polatory_gpu.h): status codes, thread-local error messages, handles.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <numeric>
#include <algorithm>
#include <set>
#include <string>
#include <unordered_map>

#include "batch.hpp"
#include "common.hpp"
#include "evaluator.hpp"
#include "model.hpp"
#include "profile.hpp"
#include "ras.hpp"
#include "rbf.cuh"
#include "solver.hpp"

namespace pgpu {
void set_device(int device);
void release_cached_memory();
void m2l_cache_stats(int64_t* bytes, int64_t* entries, int64_t* limit);
void m2l_cache_set_limit(int64_t bytes);
int direct_evaluate_noalloc(const pgpu_rbf* rbf, const double* src, int64_t ns,
                            const double* weights, const double* trg, int64_t nt, double* out,
                            cudaStream_t st, const char** msg);
}  // namespace pgpu

using namespace pgpu;

namespace {

thread_local std::string g_last_error;

template <class F>
int guarded(F&& f) {
  try {
    f();
    g_last_error.clear();
    return PGPU_OK;
  } catch (const Error& e) {
    g_last_error = e.what();
    return e.code;
  } catch (const std::bad_alloc& e) {
    g_last_error = "out of host memory";
    return PGPU_OUT_OF_MEMORY;
  } catch (const std::exception& e) {
    g_last_error = e.what();
    return PGPU_RUNTIME_ERROR;
  } catch (...) {
    g_last_error = "unknown error";
    return PGPU_RUNTIME_ERROR;
  }
}

void check_ptr(const void* p, const char* name) {
  if (p == nullptr) throw_invalid(std::string(name) + " must not be null");
}

}  // namespace

struct pgpu_evaluator {
  ModelDesc model;
  int kernel_kind = PGPU_KERNEL_VALUE;
  bool symmetric = false;
  int precision = PGPU_PRECISION_PLAIN;
  Bbox3 bbox;
  double accuracy = INFINITY;
  Index n_src = 0, n_trg = 0;
  DevBuf<double> src, trg, w, out;
  std::unique_ptr<Evaluator<double>> e64;
  std::unique_ptr<Evaluator<float>> e32;
  bool weights_set = false;
  int backend = 0;
  FarFieldConfig ff;
};

struct pgpu_interpolant {
  ModelDesc model;
  int precision = PGPU_PRECISION_PLAIN;
  bool fitted = false;
  DevBuf<double> centers, grad_centers, weights;
  std::vector<double> centers_host, grad_centers_host;
  Index mu = 0, sigma = 0;
  Bbox3 bbox;
  pgpu_fit_stats stats{};
  // Evaluation state (Interpolant::set_evaluation_bbox_impl).
  bool eval_ready = false;
  Bbox3 eval_bbox;
  double eval_accuracy = INFINITY, eval_grad_accuracy = INFINITY;
};

extern "C" {

const char* pgpu_last_error(void) { return g_last_error.c_str(); }

int pgpu_version(void) { return 100; }

int pgpu_set_device(int device) {
  return guarded([&] { set_device(device); });
}

int pgpu_release_cached_memory(void) {
  return guarded([&] { release_cached_memory(); });
}

int pgpu_profile_enable(int on) {
  return guarded([&] { profile_enable(on != 0); });
}

int pgpu_profile_reset(void) {
  return guarded([&] { profile_reset(); });
}

int pgpu_profile_report(char* buf, int64_t size) {
  return guarded([&] {
    check_ptr(buf, "buf");
    if (size <= 0) throw_invalid("size must be positive");
    std::string r = profile_report();
    size_t n = std::min<size_t>(r.size(), static_cast<size_t>(size - 1));
    std::memcpy(buf, r.data(), n);
    buf[n] = '\0';
  });
}

int pgpu_launch_count(int64_t* out) {
  return guarded([&] {
    check_ptr(out, "out");
    *out = launch_count();
  });
}

int pgpu_debug_inject(int what, int64_t after) {
  return guarded([&] {
    if (what == PGPU_INJECT_ALLOC)
      inject_alloc_failure(after);
    else if (what == PGPU_INJECT_M2L_STALL)
      inject_m2l_stall(after);
    else
      throw_invalid("unknown injection");
  });
}

int pgpu_operator_cache_stats(int64_t* bytes, int64_t* entries, int64_t* limit) {
  return guarded([&] { m2l_cache_stats(bytes, entries, limit); });
}

int pgpu_operator_cache_limit(int64_t bytes) {
  return guarded([&] {
    if (bytes < 0) throw_invalid("the limit must be >= 0");
    m2l_cache_set_limit(bytes);
  });
}

int pgpu_synchronize(void) {
  return guarded([&] { pgpu::sync(); });
}

int pgpu_stream(void** out) {
  return guarded([&] {
    check_ptr(out, "out");
    *out = reinterpret_cast<void*>(stream());
  });
}

int pgpu_rbf_evaluate(const pgpu_rbf* rbf, const double* diffs, int64_t n, double* values,
                      double* gradients, double* hessians) {
  return guarded([&] {
    check_ptr(rbf, "rbf");
    if (n < 0) throw_invalid("n must be non-negative");
    if (n > 0) check_ptr(diffs, "diffs");
    if (rbf->kind < 0 || rbf->kind >= PGPU_RBF_COUNT) throw_invalid("unknown RBF kind");
    if (hessians && !kind_has_hessian(rbf->kind)) {
      throw_runtime(std::string(rbf->kind == PGPU_RBF_CUB ? "cov_cubic" : "cov_spherical") +
                    "::evaluate_hessian_isotropic is not implemented");
    }
    const double* a = rbf->aniso;
    KParams<double> kp{rbf->params[0], rbf->params[1]};
    for (int64_t i = 0; i < n; ++i) {
      const double* d = diffs + 3 * i;
      double t[3];
      for (int r = 0; r < 3; ++r) t[r] = a[3 * r] * d[0] + a[3 * r + 1] * d[1] + a[3 * r + 2] * d[2];
      const double r2 = t[0] * t[0] + t[1] * t[1] + t[2] * t[2];
      dispatch_kind(rbf->kind, [&]<int K>() {
        if (values) values[i] = rbf_value<K>(r2, kp);
        if (gradients) {
          double c = rbf_gcoef<K>(r2, kp);
          double g[3] = {c * t[0], c * t[1], c * t[2]};
          // row vector g * A (rbf_base.hpp:45-48)
          for (int k = 0; k < 3; ++k) gradients[3 * i + k] = g[0] * a[k] + g[1] * a[3 + k] + g[2] * a[6 + k];
        }
        if (hessians) {
          double ha, hb;
          rbf_hess<K>(r2, kp, ha, hb);
          double h[9];
          for (int p = 0; p < 3; ++p)
            for (int q = 0; q < 3; ++q) h[3 * p + q] = (p == q ? ha : 0.0) + hb * t[p] * t[q];
          // A^T H A (rbf_base.hpp:50-53)
          for (int p = 0; p < 3; ++p)
            for (int q = 0; q < 3; ++q) {
              double s = 0;
              for (int u = 0; u < 3; ++u)
                for (int v = 0; v < 3; ++v) s += a[3 * u + p] * h[3 * u + v] * a[3 * v + q];
              hessians[9 * i + 3 * p + q] = s;
            }
        }
        return 0;
      });
    }
  });
}

int pgpu_rbf_cpd_order(const pgpu_rbf* rbf, int* out) {
  return guarded([&] {
    check_ptr(rbf, "rbf");
    check_ptr(out, "out");
    if (rbf->kind < 0 || rbf->kind >= PGPU_RBF_COUNT) throw_invalid("unknown RBF kind");
    *out = kind_cpd_order(rbf->kind);
  });
}

int pgpu_rbf_support_radius_isotropic(const pgpu_rbf* rbf, double* out) {
  return guarded([&] {
    check_ptr(rbf, "rbf");
    check_ptr(out, "out");
    if (rbf->kind < 0 || rbf->kind >= PGPU_RBF_COUNT) throw_invalid("unknown RBF kind");
    *out = support_radius_isotropic(rbf->kind, rbf->params);
  });
}

int pgpu_model_validate(const pgpu_model* model) {
  return guarded([&] { model_from_c(model); });
}

int pgpu_model_poly_basis_size(const pgpu_model* model, int64_t* out) {
  return guarded([&] {
    check_ptr(out, "out");
    *out = model_from_c(model).l();
  });
}

// ---- evaluator ------------------------------------------------------------------------

int pgpu_evaluator_create(const pgpu_rbf* rbf, int kernel_kind, int symmetric,
                          const double bbox[6], int precision, pgpu_evaluator** out) {
  return guarded([&] {
    check_ptr(rbf, "rbf");
    check_ptr(out, "out");
    check_ptr(bbox, "bbox");
    if (kernel_kind < PGPU_KERNEL_VALUE || kernel_kind > PGPU_KERNEL_HESSIAN)
      throw_invalid("unknown kernel kind");
    if (symmetric && (kernel_kind == PGPU_KERNEL_GRADIENT ||
                      kernel_kind == PGPU_KERNEL_GRADIENT_TRANSPOSE))
      throw_invalid("symmetric evaluators take the value or the Hessian kernel");
    pgpu_model m{};
    m.n_rbfs = 1;
    m.rbfs[0] = *rbf;
    m.poly_degree = -1;
    // Validation of the kernel alone (no polynomial constraint on a bare evaluator).
    if (rbf->kind < 0 || rbf->kind >= PGPU_RBF_COUNT) throw_invalid("unknown RBF kind");
    ModelDesc d;
    RbfDesc rd;
    rd.kind = rbf->kind;
    rd.p[0] = rbf->params[0];
    rd.p[1] = rbf->params[1];
    for (int k = 0; k < 9; ++k) rd.a[k] = rbf->aniso[k];
    if (!(det3(rd.a) > 0.0)) throw_invalid("aniso must have a positive determinant");
    d.rbfs.push_back(rd);
    d.poly_degree = -1;
    auto ev = std::make_unique<pgpu_evaluator>();
    ev->model = d;
    ev->kernel_kind = kernel_kind;
    ev->symmetric = symmetric != 0;
    ev->precision = precision;
    for (int k = 0; k < 3; ++k) {
      ev->bbox.min[k] = bbox[k];
      ev->bbox.max[k] = bbox[3 + k];
    }
    *out = ev.release();
  });
}

int pgpu_evaluator_destroy(pgpu_evaluator* ev) {
  return guarded([&] { delete ev; });
}

int pgpu_evaluator_set_accuracy(pgpu_evaluator* ev, double accuracy) {
  return guarded([&] {
    check_ptr(ev, "evaluator");
    ev->accuracy = accuracy;
    ev->e64.reset();
    ev->e32.reset();
  });
}

int pgpu_evaluator_configure(pgpu_evaluator* ev, int backend, int order, int leaf_level) {
  return guarded([&] {
    check_ptr(ev, "evaluator");
    if (backend < 0 || backend > 2) throw_invalid("unknown backend");
    if (order != 0 && order != 4 && order != 6 && order != 8) throw_invalid("order must be 4, 6 or 8");
    if (leaf_level < -1 || leaf_level > 20) throw_invalid("leaf_level out of range");
    ev->backend = backend;
    ev->ff.order = order;
    ev->ff.leaf_level = leaf_level;
    ev->e64.reset();
    ev->e32.reset();
  });
}

namespace {
// Inputs per source (km) and outputs per target (kn) of a kernel kind: gradient sources carry
// three weights (GradientKernel, HessianKernel: km = 3, fmm/gradient_kernel.hpp:28-29), gradient
// targets receive three outputs (GradientTransposeKernel, HessianKernel: kn = 3).
bool grad_sources(int kind) {
  return kind == PGPU_KERNEL_GRADIENT || kind == PGPU_KERNEL_HESSIAN;
}
bool grad_targets(int kind) {
  return kind == PGPU_KERNEL_GRADIENT_TRANSPOSE || kind == PGPU_KERNEL_HESSIAN;
}

// The kernel kinds are the blocks of one Evaluator: value or gradient point sets on either
// side (interpolation/evaluator.hpp:97-124 wires a_, f_, ft_, h_ the same way).
void rebuild(pgpu_evaluator* ev) {
  auto wire = [ev](auto& e) {
    e.set_backend(ev->backend);
    e.set_far_field(ev->ff);
    const bool gs = grad_sources(ev->kernel_kind), gt = grad_targets(ev->kernel_kind);
    if (ev->symmetric) {
      if (gs) e.set_points(nullptr, 0, ev->src.data(), ev->n_src);
      else e.set_points(ev->src.data(), ev->n_src, nullptr, 0);
      return;
    }
    if (gs) e.set_sources(nullptr, 0, ev->src.data(), ev->n_src);
    else e.set_sources(ev->src.data(), ev->n_src, nullptr, 0);
    if (gt) e.set_targets(nullptr, 0, ev->trg.data(), ev->n_trg);
    else e.set_targets(ev->trg.data(), ev->n_trg, nullptr, 0);
  };
  if (ev->precision == PGPU_PRECISION_PLAIN) {
    ev->e64 = std::make_unique<Evaluator<double>>(ev->model, ev->bbox, ev->accuracy, ev->accuracy);
    wire(*ev->e64);
  } else {
    ev->e32 = std::make_unique<Evaluator<float>>(ev->model, ev->bbox, ev->accuracy, ev->accuracy);
    wire(*ev->e32);
  }
}
}  // namespace

int pgpu_evaluator_set_source_points(pgpu_evaluator* ev, const double* points, int64_t n) {
  return guarded([&] {
    check_ptr(ev, "evaluator");
    if (ev->symmetric) throw_invalid("symmetric evaluators take set_points");
    if (n < 0) throw_invalid("n must be non-negative");
    copy_in(ev->src, points, 3 * n);
    ev->n_src = n;
    ev->e64.reset();
    ev->e32.reset();
    ev->weights_set = false;
    if (!device_all_finite(ev->src.data(), 3 * n)) {
      ev->n_src = 0;
      throw_invalid("points must be finite");
    }
  });
}

int pgpu_evaluator_set_target_points(pgpu_evaluator* ev, const double* points, int64_t n) {
  return guarded([&] {
    check_ptr(ev, "evaluator");
    if (ev->symmetric) throw_invalid("symmetric evaluators take set_points");
    if (n < 0) throw_invalid("n must be non-negative");
    copy_in(ev->trg, points, 3 * n);
    ev->n_trg = n;
    ev->e64.reset();
    ev->e32.reset();
    if (!device_all_finite(ev->trg.data(), 3 * n)) {
      ev->n_trg = 0;
      throw_invalid("points must be finite");
    }
  });
}

int pgpu_evaluator_set_points(pgpu_evaluator* ev, const double* points, int64_t n) {
  return guarded([&] {
    check_ptr(ev, "evaluator");
    if (!ev->symmetric) throw_invalid("set_points needs a symmetric evaluator");
    if (n < 0) throw_invalid("n must be non-negative");
    copy_in(ev->src, points, 3 * n);
    ev->n_src = ev->n_trg = n;
    ev->e64.reset();
    ev->e32.reset();
    ev->weights_set = false;
    if (!device_all_finite(ev->src.data(), 3 * n)) {
      ev->n_src = ev->n_trg = 0;
      throw_invalid("points must be finite");
    }
  });
}

int pgpu_evaluator_set_weights(pgpu_evaluator* ev, const double* weights, int64_t n) {
  return guarded([&] {
    check_ptr(ev, "evaluator");
    if (n != (grad_sources(ev->kernel_kind) ? 3 : 1) * ev->n_src)
      throw_invalid("weights must have km * n_sources entries");
    copy_in(ev->w, weights, n);
    ev->weights_set = true;
  });
}

int pgpu_evaluator_evaluate(pgpu_evaluator* ev, double* out, int64_t n) {
  return guarded([&] {
    check_ptr(ev, "evaluator");
    if (n != (grad_targets(ev->kernel_kind) ? 3 : 1) * ev->n_trg)
      throw_invalid("out must have kn * n_targets entries");
    if (!ev->weights_set) throw_runtime("weights have not been set");
    if (!ev->e64 && !ev->e32) rebuild(ev);
    ev->out.resize(std::max<int64_t>(n, 1));
    if (ev->e64) {
      ev->e64->set_weights(ev->w.data());
      ev->e64->evaluate(ev->out.data(), false);
    } else {
      ev->e32->set_weights(ev->w.data());
      ev->e32->evaluate(ev->out.data(), false);
    }
    copy_out(out, ev->out.data(), n);
  });
}

int pgpu_direct_evaluate_noalloc(const pgpu_rbf* rbf, const double* src_points, int64_t n_src,
                                 const double* weights, const double* trg_points, int64_t n_trg,
                                 double* out, void* stream) {
  // No device allocation on any path (see noalloc.cu); the message string is only written when
  // the call fails.
  const char* msg = nullptr;
  int rc = direct_evaluate_noalloc(rbf, src_points, n_src, weights, trg_points, n_trg, out,
                                   static_cast<cudaStream_t>(stream), &msg);
  if (rc != PGPU_OK) g_last_error = msg ? msg : "allocation-free evaluation failed";
  else g_last_error.clear();
  return rc;
}

namespace {
void check_fit_args(const ModelDesc& m, int64_t mu, int64_t sigma, double tol, double grad_tol,
                    int max_iter, double acc, double grad_acc);
}  // namespace

int pgpu_fit_batch(const pgpu_model* model, int precision, pgpu_fit_problem* problems,
                   int64_t n_problems, int n_workers) {
  int rc = PGPU_OK;
  int status = guarded([&] {
    ModelDesc m = model_from_c(model);
    if (n_problems < 0) throw_invalid("n_problems must be non-negative");
    if (n_problems > 0) check_ptr(problems, "problems");
    if (precision != PGPU_PRECISION_PLAIN && precision != PGPU_PRECISION_MIXED)
      throw_invalid("unknown precision");
    for (int64_t i = 0; i < n_problems; ++i) {
      auto& p = problems[i];
      check_fit_args(m, p.n, 0, p.tolerance, INFINITY, p.max_iter, INFINITY, INFINITY);
      check_ptr(p.points, "points");
      check_ptr(p.values, "values");
      p.status = PGPU_OK;
      p.iterations = 0;
    }
    int device = 0;
    PGPU_CUDA(cudaGetDevice(&device));
    std::string first;
    rc = run_batch(m, precision, problems, n_problems, n_workers, device, &first);
    if (rc != PGPU_OK) throw Error(rc, first + " (each problem's status is set)");
  });
  return status;
}

// ---- interpolant ----------------------------------------------------------------------

int pgpu_krylov_fgmres_dense(int64_t n, const double* op, const double* pc, const double* rhs,
                             const double* x0, int iters, double* solutions, double* rel_residuals) {
  return guarded([&] {
    check_ptr(op, "op");
    check_ptr(rhs, "rhs");
    if (iters > 0) {
      check_ptr(solutions, "solutions");
      check_ptr(rel_residuals, "rel_residuals");
    }
    krylov_fgmres_dense(n, op, pc, rhs, x0, iters, solutions, rel_residuals);
  });
}

int pgpu_ras_domain_solve(const pgpu_model* model, const double* points, int64_t n,
                          const int64_t* order, const unsigned char* inner, int coarse,
                          int use_inverse, int precision, const double* rhs, double* out) {
  return guarded([&] {
    ModelDesc m = model_from_c(model);
    if (n <= 0) throw_invalid("n must be positive");
    check_ptr(points, "points");
    check_ptr(order, "order");
    check_ptr(inner, "inner");
    check_ptr(rhs, "rhs");
    check_ptr(out, "out");
    if (precision != PGPU_PRECISION_PLAIN && precision != PGPU_PRECISION_MIXED)
      throw_invalid("unknown precision");
    ras_domain_solve(m, points, n, order, inner, coarse != 0, use_inverse != 0,
                     precision == PGPU_PRECISION_MIXED, rhs, out);
  });
}

int pgpu_interpolant_create(const pgpu_model* model, pgpu_interpolant** out) {
  return guarded([&] {
    check_ptr(out, "out");
    auto it = std::make_unique<pgpu_interpolant>();
    it->model = model_from_c(model);
    *out = it.release();
  });
}

int pgpu_interpolant_destroy(pgpu_interpolant* it) {
  return guarded([&] { delete it; });
}

int pgpu_interpolant_set_precision(pgpu_interpolant* it, int precision) {
  return guarded([&] {
    check_ptr(it, "interpolant");
    if (precision != PGPU_PRECISION_PLAIN && precision != PGPU_PRECISION_MIXED)
      throw_invalid("unknown precision");
    it->precision = precision;
  });
}

namespace {

std::vector<double> host_copy(const double* p, size_t n) {
  std::vector<double> v(n);
  if (n == 0) return v;
  if (is_device_pointer(p)) {
    PGPU_CUDA(cudaMemcpy(v.data(), p, n * sizeof(double), cudaMemcpyDeviceToHost));
  } else {
    std::memcpy(v.data(), p, n * sizeof(double));
  }
  return v;
}

// Interpolant::check_* (interpolant.hpp:275-315).
void check_fit_args(const ModelDesc& m, int64_t mu, int64_t sigma, double tol, double grad_tol,
                    int max_iter, double acc, double grad_acc) {
  const int l = m.l();
  if (mu < 0 || sigma < 0) throw_invalid("point counts must be non-negative");
  if (!(m.poly_degree == 1 && mu == 1 && sigma >= 1) && mu < l)
    throw_invalid("points.rows() must be greater than or equal to " + std::to_string(l));
  if (!(tol > 0.0)) throw_invalid("tolerance must be positive");
  if (!(grad_tol > 0.0)) throw_invalid("grad_tolerance must be positive");
  if (max_iter < 0) throw_invalid("max_iter must be nonnegative");
  if (!(acc > 0.0)) throw_invalid("accuracy must be positive");
  if (!(grad_acc > 0.0)) throw_invalid("grad_accuracy must be positive");
}

}  // namespace

int pgpu_interpolant_fit(pgpu_interpolant* it, const double* points, int64_t mu,
                         const double* grad_points, int64_t sigma, const double* values,
                         double tolerance, double grad_tolerance, int max_iter, double accuracy,
                         double grad_accuracy, const pgpu_interpolant* initial) {
  return guarded([&] {
    check_ptr(it, "interpolant");
    check_fit_args(it->model, mu, sigma, tolerance, grad_tolerance, max_iter, accuracy,
                   grad_accuracy);
    if (mu > 0) check_ptr(points, "points");
    if (sigma > 0) check_ptr(grad_points, "grad_points");
    check_ptr(values, "values");
    const int l = it->model.l();
    const double t_in = wall_seconds();
    auto pts = host_copy(points, 3 * mu);
    auto gpts = host_copy(grad_points, 3 * sigma);
    auto vals = host_copy(values, mu + 3 * sigma);
    if (std::getenv("PGPU_VERBOSE"))
      std::printf("fit: inputs to host %.3f s\n", wall_seconds() - t_in);

    std::vector<double> init;
    if (initial != nullptr && initial->fitted) {
      // Interpolant::build_initial_weights (interpolant.hpp:232-273): copy the weights of the
      // centres that reappear (exact coordinate match) and the polynomial coefficients.
      init.assign(mu + 3 * sigma + l, 0.0);
      const bool same_model = initial->model.poly_degree == it->model.poly_degree &&
                              initial->model.nugget == it->model.nugget &&
                              initial->model.rbfs.size() == it->model.rbfs.size();
      if (same_model) {
        auto iw = initial->weights.to_host();
        std::unordered_map<std::string, Index> pos;
        for (Index i = 0; i < initial->mu; ++i)
          pos.emplace(std::string(reinterpret_cast<const char*>(&initial->centers_host[3 * i]),
                                  3 * sizeof(double)),
                      i);
        for (Index i = 0; i < mu; ++i) {
          auto f = pos.find(std::string(reinterpret_cast<const char*>(&pts[3 * i]), 3 * sizeof(double)));
          if (f != pos.end()) init[i] = iw[f->second];
        }
        // Gradient centres: their three weights (interpolant.hpp:262-268).
        std::unordered_map<std::string, Index> gpos;
        for (Index i = 0; i < initial->sigma; ++i)
          gpos.emplace(std::string(reinterpret_cast<const char*>(&initial->grad_centers_host[3 * i]),
                                   3 * sizeof(double)),
                       i);
        for (Index i = 0; i < sigma; ++i) {
          auto f = gpos.find(std::string(reinterpret_cast<const char*>(&gpts[3 * i]), 3 * sizeof(double)));
          if (f != gpos.end())
            for (int c = 0; c < 3; ++c) init[mu + 3 * i + c] = iw[initial->mu + 3 * f->second + c];
        }
        for (int k = 0; k < l; ++k) init[mu + 3 * sigma + k] = iw[iw.size() - l + k];
      }
    }

    it->fitted = false;
    FitRequest req;
    req.model = &it->model;
    req.points_host = pts.data();
    req.mu = mu;
    req.grad_points_host = gpts.data();
    req.sigma = sigma;
    req.values_host = vals.data();
    req.tolerance = tolerance;
    req.grad_tolerance = grad_tolerance;
    req.max_iter = max_iter;
    req.accuracy = accuracy;
    req.grad_accuracy = grad_accuracy;
    req.initial_weights = init.empty() ? nullptr : init.data();
    req.precision = it->precision;
    req.verbose = std::getenv("PGPU_VERBOSE") != nullptr;
    FitResult r = fit(req);

    it->weights.upload(r.weights);
    it->centers.upload(pts);
    it->grad_centers.upload(gpts);
    it->centers_host = std::move(pts);
    it->mu = mu;
    it->sigma = sigma;
    it->bbox = Bbox3::from_host_points(it->centers_host.data(), mu)
                   .hull(Bbox3::from_host_points(gpts.data(), sigma));
    it->grad_centers_host = std::move(gpts);
    it->stats.iterations = r.iterations;
    it->stats.levels = r.levels;
    it->stats.residual = r.residual;
    it->stats.grad_residual = r.grad_residual;
    it->stats.setup_seconds = r.setup_seconds;
    it->stats.solve_seconds = r.solve_seconds;
    it->stats.n_domains = r.n_domains;
    it->stats.precision_used = r.precision_used;
    it->stats.fell_back = r.fell_back ? 1 : 0;
    it->fitted = true;
    it->eval_ready = false;
  });
}

namespace {
void throw_if_not_fitted(const pgpu_interpolant* it) {
  check_ptr(it, "interpolant");
  if (!it->fitted) throw_runtime("interpolant has not been fitted");
}

void run_evaluate(pgpu_interpolant* it, const double* points, int64_t m, const double* grad_points,
                  int64_t mg, double* out) {
  if (m < 0 || mg < 0) throw_invalid("point counts must be non-negative");
  if (m > 0) check_ptr(points, "points");
  if (mg > 0) check_ptr(grad_points, "grad_points");
  if (m + 3 * mg > 0) check_ptr(out, "out");
  DevBuf<double> q, gq, o;
  copy_in(q, points, 3 * m);
  copy_in(gq, grad_points, 3 * mg);
  o.resize(std::max<int64_t>(m + 3 * mg, 1));
  EvaluateRequest req;
  req.model = &it->model;
  req.centers_dev = it->centers.data();
  req.mu = it->mu;
  req.grad_centers_dev = it->grad_centers.data();
  req.sigma = it->sigma;
  req.weights_dev = it->weights.data();
  req.bbox = it->eval_bbox;
  req.points_dev = q.data();
  req.m = m;
  req.grad_points_dev = gq.data();
  req.mg = mg;
  req.accuracy = it->eval_accuracy;
  req.grad_accuracy = it->eval_grad_accuracy;
  req.precision = it->precision;
  req.out_dev = o.data();
  evaluate(req);
  copy_out(out, o.data(), m + 3 * mg);
}
}  // namespace

int pgpu_interpolant_set_evaluation_bbox(pgpu_interpolant* it, const double bbox[6],
                                         double accuracy, double grad_accuracy) {
  return guarded([&] {
    throw_if_not_fitted(it);
    check_ptr(bbox, "bbox");
    Bbox3 b;
    for (int k = 0; k < 3; ++k) {
      b.min[k] = bbox[k];
      b.max[k] = bbox[3 + k];
    }
    it->eval_bbox = b.hull(it->bbox);
    it->eval_accuracy = accuracy;
    it->eval_grad_accuracy = grad_accuracy;
    it->eval_ready = true;
  });
}

int pgpu_interpolant_evaluate(pgpu_interpolant* it, const double* points, int64_t m,
                              const double* grad_points, int64_t mg, double accuracy,
                              double grad_accuracy, double* out) {
  return guarded([&] {
    throw_if_not_fitted(it);
    if (!(accuracy > 0.0)) throw_invalid("accuracy must be positive");
    if (!(grad_accuracy > 0.0)) throw_invalid("grad_accuracy must be positive");
    auto bbox_of = [](const double* p, int64_t n) {
      if (n == 0) return Bbox3{};
      if (is_device_pointer(p)) return bbox_of_device_points(p, n);
      return Bbox3::from_host_points(p, n);
    };
    Bbox3 b = bbox_of(points, m).hull(bbox_of(grad_points, mg));
    it->eval_bbox = b.hull(it->bbox);
    it->eval_accuracy = accuracy;
    it->eval_grad_accuracy = grad_accuracy;
    it->eval_ready = true;
    run_evaluate(it, points, m, grad_points, mg, out);
  });
}

int pgpu_interpolant_evaluate_impl(pgpu_interpolant* it, const double* points, int64_t m,
                                   const double* grad_points, int64_t mg, double* out) {
  return guarded([&] {
    throw_if_not_fitted(it);
    if (!it->eval_ready) {
      it->eval_bbox = it->bbox;
      it->eval_ready = true;
    }
    run_evaluate(it, points, m, grad_points, mg, out);
  });
}

int pgpu_interpolant_evaluate_lattice(pgpu_interpolant* it, const double lc_origin[3],
                                      const double basis[9], const int32_t* lcs, int64_t n,
                                      double isovalue, double* out) {
  return guarded([&] {
    throw_if_not_fitted(it);
    check_ptr(lc_origin, "lc_origin");
    check_ptr(basis, "basis");
    if (n < 0) throw_invalid("n must be non-negative");
    if (n == 0) return;
    check_ptr(lcs, "lcs");
    check_ptr(out, "out");
    DevBuf<int32_t> dl(static_cast<size_t>(3 * n));
    const bool dev = is_device_pointer(lcs);
    PGPU_CUDA(cudaMemcpyAsync(dl.data(), lcs, 3 * n * sizeof(int32_t),
                              dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, stream()));
    if (!dev) pgpu::sync();
    DevBuf<double> pts(static_cast<size_t>(3 * n)), vals(static_cast<size_t>(n));
    lattice_positions(lc_origin, basis, dl.data(), n, pts.data());
    if (!it->eval_ready) {
      it->eval_bbox = it->bbox;
      it->eval_ready = true;
    }
    run_evaluate(it, pts.data(), n, nullptr, 0, vals.data());
    subtract_scalar(vals.data(), n, isovalue);
    copy_out(out, vals.data(), n);
  });
}

int pgpu_interpolant_is_fitted(const pgpu_interpolant* it, int* out) {
  return guarded([&] {
    check_ptr(it, "interpolant");
    check_ptr(out, "out");
    *out = it->fitted ? 1 : 0;
  });
}

int pgpu_interpolant_num_weights(const pgpu_interpolant* it, int64_t* out) {
  return guarded([&] {
    throw_if_not_fitted(it);
    check_ptr(out, "out");
    *out = static_cast<int64_t>(it->weights.size());
  });
}

int pgpu_interpolant_weights(const pgpu_interpolant* it, double* out, int64_t n) {
  return guarded([&] {
    throw_if_not_fitted(it);
    if (n != static_cast<int64_t>(it->weights.size())) throw_invalid("wrong weights length");
    copy_out(out, it->weights.data(), n);
  });
}

int pgpu_interpolant_num_centers(const pgpu_interpolant* it, int64_t* mu, int64_t* sigma) {
  return guarded([&] {
    throw_if_not_fitted(it);
    if (mu) *mu = it->mu;
    if (sigma) *sigma = it->sigma;
  });
}

int pgpu_interpolant_centers(const pgpu_interpolant* it, double* centers, double* grad_centers) {
  return guarded([&] {
    throw_if_not_fitted(it);
    if (centers && it->mu) copy_out(centers, it->centers.data(), 3 * it->mu);
    if (grad_centers && it->sigma) copy_out(grad_centers, it->grad_centers.data(), 3 * it->sigma);
  });
}

int pgpu_interpolant_bbox(const pgpu_interpolant* it, double bbox[6]) {
  return guarded([&] {
    throw_if_not_fitted(it);
    check_ptr(bbox, "bbox");
    for (int k = 0; k < 3; ++k) {
      bbox[k] = it->bbox.min[k];
      bbox[3 + k] = it->bbox.max[k];
    }
  });
}

int pgpu_interpolant_fit_stats(const pgpu_interpolant* it, pgpu_fit_stats* out) {
  return guarded([&] {
    throw_if_not_fitted(it);
    check_ptr(out, "out");
    *out = it->stats;
  });
}

}  // extern "C"

// ---- serving ----------------------------------------------------------------------------

namespace pgpu {
int server_create(int n_workers, int64_t budget, pgpu_server** out);
void server_destroy(pgpu_server* s);
int64_t server_estimate(const pgpu_request& r);
void server_submit(pgpu_server* s, const pgpu_request& r, int64_t* ticket);
bool server_poll(pgpu_server* s, int64_t ticket, bool block, int* status, double* latency,
                 std::string* msg);
void server_stats(pgpu_server* s, pgpu_server_stats* o);
}  // namespace pgpu

namespace {

void check_request(const pgpu_request* r) {
  check_ptr(r, "request");
  if (r->kind != PGPU_REQUEST_FIT && r->kind != PGPU_REQUEST_EVALUATE)
    throw_invalid("unknown request kind");
  if (r->precision != PGPU_PRECISION_PLAIN && r->precision != PGPU_PRECISION_MIXED)
    throw_invalid("unknown precision");
  if (r->n < 0) throw_invalid("n must be non-negative");
  if (r->n > 0) check_ptr(r->points, "points");
  if (r->kind == PGPU_REQUEST_FIT) {
    ModelDesc m = model_from_c(r->model);
    check_fit_args(m, r->n, 0, r->tolerance, INFINITY, r->max_iter, INFINITY, INFINITY);
    check_ptr(r->values, "values");
  } else if (r->n > 0) {
    check_ptr(r->out, "out");
  }
}

}  // namespace

int pgpu_server_create(int n_workers, int64_t hbm_budget_bytes, pgpu_server** out) {
  return guarded([&] {
    check_ptr(out, "out");
    if (n_workers < 0) throw_invalid("n_workers must be non-negative");
    if (hbm_budget_bytes < 0) throw_invalid("hbm_budget_bytes must be non-negative");
    server_create(n_workers, hbm_budget_bytes, out);
  });
}

int pgpu_server_destroy(pgpu_server* s) {
  return guarded([&] {
    if (s) server_destroy(s);
  });
}

int pgpu_server_submit(pgpu_server* s, const pgpu_request* req, int64_t* ticket) {
  return guarded([&] {
    check_ptr(s, "server");
    check_ptr(ticket, "ticket");
    check_request(req);
    server_submit(s, *req, ticket);
  });
}

int pgpu_server_poll(pgpu_server* s, int64_t ticket, int* done, int* status, double* latency) {
  std::string msg;
  int rc = guarded([&] {
    check_ptr(s, "server");
    check_ptr(done, "done");
    int st = PGPU_OK;
    double lat = 0;
    *done = server_poll(s, ticket, false, &st, &lat, &msg) ? 1 : 0;
    if (status) *status = st;
    if (latency) *latency = lat;
  });
  if (rc == PGPU_OK && !msg.empty()) g_last_error = msg;
  return rc;
}

int pgpu_server_wait(pgpu_server* s, int64_t ticket, int* status, double* latency) {
  std::string msg;
  int rc = guarded([&] {
    check_ptr(s, "server");
    int st = PGPU_OK;
    double lat = 0;
    server_poll(s, ticket, true, &st, &lat, &msg);
    if (status) *status = st;
    if (latency) *latency = lat;
  });
  if (rc == PGPU_OK && !msg.empty()) g_last_error = msg;
  return rc;
}

int pgpu_server_stats_get(pgpu_server* s, pgpu_server_stats* out) {
  return guarded([&] {
    check_ptr(s, "server");
    check_ptr(out, "out");
    server_stats(s, out);
  });
}

int64_t pgpu_server_estimate_bytes(const pgpu_request* req) {
  if (!req) return -1;
  return server_estimate(*req);
}

// ---- save / load (the reference's binary format) -------------------------------------------
// common/io.hpp:31-187 with Write<Interpolant> (interpolant.hpp:345-367), Write<Model>
// (model.hpp:304-320), Write<Rbf> (rbf/rbf_io.hpp), Write<Bbox> (geometry/bbox3d.hpp:82-96):
// trivially copyable values as their bytes; std::string and std::vector as a size_t count and
// the elements; dynamic Eigen matrices as their Index row count (fixed columns are not written)
// and the data in storage order (points row-major); fixed-size matrices as their data
// (anisotropy row-major). Little-endian, as on both hosts.

namespace {

const char* const kShortNames[PGPU_RBF_COUNT] = {"bh2", "bh3", "cub", "exp", "gau", "gc3",
                                                 "gc5", "gc7", "gc9", "sph", "sp3", "sp5",
                                                 "sp7", "sp9", "th2", "th3"};

struct Out {
  std::vector<char> b;
  template <class V>
  void put(const V& v) {
    const char* p = reinterpret_cast<const char*>(&v);
    b.insert(b.end(), p, p + sizeof(V));
  }
  void put_doubles(const double* p, size_t n) {
    const char* c = reinterpret_cast<const char*>(p);
    b.insert(b.end(), c, c + n * sizeof(double));
  }
};

struct In {
  const std::vector<char>& b;
  size_t pos = 0;
  template <class V>
  V get() {
    if (pos + sizeof(V) > b.size()) throw_runtime("unexpected end of the interpolant file");
    V v;
    std::memcpy(&v, b.data() + pos, sizeof(V));
    pos += sizeof(V);
    return v;
  }
  void get_doubles(double* p, size_t n) {
    if (pos + n * sizeof(double) > b.size()) throw_runtime("unexpected end of the interpolant file");
    std::memcpy(p, b.data() + pos, n * sizeof(double));
    pos += n * sizeof(double);
  }
};

std::vector<char> serialize(const pgpu_interpolant* it) {
  Out o;
  o.put(static_cast<uint64_t>(it->model.rbfs.size()));
  for (const auto& r : it->model.rbfs) {
    const std::string name = kShortNames[r.kind];
    o.put(static_cast<uint64_t>(name.size()));
    o.b.insert(o.b.end(), name.begin(), name.end());
    o.put(static_cast<uint64_t>(2));
    o.put_doubles(r.p, 2);
    o.put_doubles(r.a, 9);
  }
  o.put(static_cast<int32_t>(it->model.poly_degree));
  o.put(it->model.nugget);
  o.put(static_cast<uint8_t>(it->fitted ? 1 : 0));
  o.put(static_cast<int64_t>(it->mu));
  o.put_doubles(it->centers_host.data(), 3 * static_cast<size_t>(it->mu));
  std::vector<double> g(3 * static_cast<size_t>(it->sigma));
  if (it->sigma > 0) copy_out(g.data(), it->grad_centers.data(), g.size());
  o.put(static_cast<int64_t>(it->sigma));
  o.put_doubles(g.data(), g.size());
  o.put_doubles(it->bbox.min, 3);
  o.put_doubles(it->bbox.max, 3);
  std::vector<double> w(it->fitted ? it->weights.size() : 0);
  if (!w.empty()) copy_out(w.data(), it->weights.data(), w.size());
  o.put(static_cast<int64_t>(w.size()));
  o.put_doubles(w.data(), w.size());
  return std::move(o.b);
}

std::unique_ptr<pgpu_interpolant> deserialize(const std::vector<char>& bytes) {
  In in{bytes};
  pgpu_model m{};
  const uint64_t n_rbfs = in.get<uint64_t>();
  if (n_rbfs < 1 || n_rbfs > 4) throw_runtime("unsupported number of RBFs in the interpolant file");
  m.n_rbfs = static_cast<int32_t>(n_rbfs);
  for (uint64_t k = 0; k < n_rbfs; ++k) {
    const uint64_t len = in.get<uint64_t>();
    if (len > 16) throw_runtime("bad RBF name in the interpolant file");
    std::string name(len, '\0');
    for (auto& ch : name) ch = in.get<char>();
    int kind = -1;
    for (int q = 0; q < PGPU_RBF_COUNT; ++q)
      if (name == kShortNames[q]) kind = q;
    if (kind < 0) throw_runtime("unknown RBF '" + name + "' in the interpolant file");
    const uint64_t np = in.get<uint64_t>();
    if (np > 2) throw_runtime("bad RBF parameters in the interpolant file");
    m.rbfs[k].kind = kind;
    m.rbfs[k].params[0] = 1.0;
    m.rbfs[k].params[1] = 0.0;
    in.get_doubles(m.rbfs[k].params, np);
    in.get_doubles(m.rbfs[k].aniso, 9);
  }
  m.poly_degree = in.get<int32_t>();
  m.nugget = in.get<double>();
  auto it = std::make_unique<pgpu_interpolant>();
  it->model = model_from_c(&m);
  const bool fitted = in.get<uint8_t>() != 0;
  const int64_t mu = in.get<int64_t>();
  if (mu < 0) throw_runtime("bad point count in the interpolant file");
  std::vector<double> pts(3 * static_cast<size_t>(mu));
  in.get_doubles(pts.data(), pts.size());
  const int64_t sigma = in.get<int64_t>();
  if (sigma < 0) throw_runtime("bad point count in the interpolant file");
  std::vector<double> gpts(3 * static_cast<size_t>(sigma));
  in.get_doubles(gpts.data(), gpts.size());
  in.get_doubles(it->bbox.min, 3);
  in.get_doubles(it->bbox.max, 3);
  const int64_t nw = in.get<int64_t>();
  if (nw < 0) throw_runtime("bad weight count in the interpolant file");
  std::vector<double> w(static_cast<size_t>(nw));
  in.get_doubles(w.data(), w.size());
  if (fitted) {
    if (nw != mu + 3 * sigma + it->model.l())
      throw_runtime("the weights of the interpolant file do not match its centers");
    it->weights.upload(w);
    it->centers.upload(pts);
    it->grad_centers.upload(gpts);
    pgpu::sync();
  }
  it->centers_host = std::move(pts);
  it->grad_centers_host = std::move(gpts);
  it->mu = mu;
  it->sigma = sigma;
  it->fitted = fitted;
  return it;
}

}  // namespace

int pgpu_interpolant_save(const pgpu_interpolant* it, const char* filename) {
  return guarded([&] {
    check_ptr(it, "interpolant");
    check_ptr(filename, "filename");
    const std::vector<char> bytes = serialize(it);
    std::FILE* f = std::fopen(filename, "wb");
    if (!f) throw_runtime(std::string("cannot open file '") + filename + "'");
    const size_t wrote = std::fwrite(bytes.data(), 1, bytes.size(), f);
    const int closed = std::fclose(f);
    if (wrote != bytes.size() || closed != 0)
      throw_runtime(std::string("cannot write file '") + filename + "'");
  });
}

int pgpu_interpolant_load(const char* filename, pgpu_interpolant** out) {
  return guarded([&] {
    check_ptr(filename, "filename");
    check_ptr(out, "out");
    std::FILE* f = std::fopen(filename, "rb");
    if (!f) throw_runtime(std::string("cannot open file '") + filename + "'");
    std::vector<char> bytes;
    char buf[1 << 16];
    size_t got;
    while ((got = std::fread(buf, 1, sizeof(buf), f)) > 0) bytes.insert(bytes.end(), buf, buf + got);
    std::fclose(f);
    *out = deserialize(bytes).release();
  });
}

// ---- incremental fit (interpolation/incremental_fitter.hpp:46-183) --------------------------

namespace {

// DistanceFilter::filter (point_cloud/distance_filter.hpp:31-65): walking the indices in order,
// a point not yet removed removes every other point of the full set within the distance. A
// uniform grid with the distance as its cell size stands in for the kd-tree radius search.
std::vector<char> distance_filter_keep(const std::vector<double>& pts, double distance,
                                       const std::vector<Index>& indices) {
  const Index n = static_cast<Index>(pts.size() / 3);
  std::vector<char> removed(n, 0), keep(n, 0);
  if (n == 0) return keep;
  double mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (Index i = 0; i < n; ++i)
    for (int k = 0; k < 3; ++k) {
      mn[k] = std::min(mn[k], pts[3 * i + k]);
      mx[k] = std::max(mx[k], pts[3 * i + k]);
    }
  int64_t dims[3];
  for (int k = 0; k < 3; ++k)
    dims[k] = std::max<int64_t>(1, std::min<int64_t>(1 << 10, static_cast<int64_t>((mx[k] - mn[k]) / distance) + 1));
  auto cell_of = [&](Index i, int k) {
    return std::min<int64_t>(dims[k] - 1, static_cast<int64_t>((pts[3 * i + k] - mn[k]) / distance));
  };
  std::unordered_map<int64_t, std::vector<Index>> grid;
  auto key = [&](int64_t x, int64_t y, int64_t z) { return (x * dims[1] + y) * dims[2] + z; };
  for (Index i = 0; i < n; ++i) grid[key(cell_of(i, 0), cell_of(i, 1), cell_of(i, 2))].push_back(i);
  const double d2max = distance * distance;
  for (Index i : indices) {
    if (removed[i]) continue;
    const int64_t cx = cell_of(i, 0), cy = cell_of(i, 1), cz = cell_of(i, 2);
    for (int64_t x = std::max<int64_t>(0, cx - 1); x <= std::min(dims[0] - 1, cx + 1); ++x)
      for (int64_t y = std::max<int64_t>(0, cy - 1); y <= std::min(dims[1] - 1, cy + 1); ++y)
        for (int64_t z = std::max<int64_t>(0, cz - 1); z <= std::min(dims[2] - 1, cz + 1); ++z) {
          auto f = grid.find(key(x, y, z));
          if (f == grid.end()) continue;
          for (Index j : f->second) {
            if (j == i) continue;
            double d2 = 0;
            for (int k = 0; k < 3; ++k) {
              const double d = pts[3 * i + k] - pts[3 * j + k];
              d2 += d * d;
            }
            if (d2 <= d2max) removed[j] = 1;
          }
        }
  }
  for (Index i : indices)
    if (!removed[i]) keep[i] = 1;
  return keep;
}

}  // namespace

int pgpu_interpolant_fit_incrementally(pgpu_interpolant* it, const double* points, int64_t mu_full,
                                       const double* grad_points, int64_t sigma_full,
                                       const double* values, double tolerance,
                                       double grad_tolerance, int max_iter, double accuracy,
                                       double grad_accuracy) {
  return guarded([&] {
    check_ptr(it, "interpolant");
    check_fit_args(it->model, mu_full, sigma_full, tolerance, grad_tolerance, max_iter, accuracy,
                   grad_accuracy);
    if (sigma_full > 0) throw Error(PGPU_NOT_IMPLEMENTED, "gradient data points are not supported yet");
    if (mu_full > 0) check_ptr(points, "points");
    check_ptr(values, "values");
    const int l = it->model.l();
    const auto pts = host_copy(points, 3 * mu_full);
    const auto vals = host_copy(values, mu_full);
    const Bbox3 bbox = Bbox3::from_host_points(pts.data(), mu_full);
    const bool verbose_out = std::getenv("PGPU_VERBOSE") != nullptr;
    constexpr double kMinDistance = 1.0842021724855044e-19;  // DistanceFilter::kMinDistance
    double diag = 0;
    for (int k = 0; k < 3; ++k) diag += (bbox.max[k] - bbox.min[k]) * (bbox.max[k] - bbox.min[k]);
    double filtering_distance = std::max(std::sqrt(diag), kMinDistance);

    std::vector<Index> centers;
    std::vector<double> weights(l, 0.0);
    std::vector<char> is_center(mu_full, 0);
    it->fitted = false;
    while (true) {
      const Index mu = static_cast<Index>(centers.size());
      std::vector<double> cp(3 * mu), cv(mu);
      for (Index i = 0; i < mu; ++i) {
        for (int k = 0; k < 3; ++k) cp[3 * i + k] = pts[3 * centers[i] + k];
        cv[i] = vals[centers[i]];
      }
      if (verbose_out) std::printf("Number of RBF centers: %ld / %ld\n", static_cast<long>(mu), static_cast<long>(mu_full));
      if (mu >= l && mu > 0) {
        FitRequest req;
        req.model = &it->model;
        req.points_host = cp.data();
        req.mu = mu;
        req.values_host = cv.data();
        req.tolerance = tolerance;
        req.grad_tolerance = grad_tolerance;
        req.max_iter = max_iter;
        req.accuracy = accuracy;
        req.grad_accuracy = grad_accuracy;
        req.initial_weights = weights.data();
        req.precision = it->precision;
        req.verbose = verbose_out;
        weights = fit(req).weights;
      }
      if (mu == mu_full) break;

      // Residuals at the remaining points, sorted ascending (stable in index order).
      std::vector<Index> rest;
      for (Index i = 0; i < mu_full; ++i)
        if (!is_center[i]) rest.push_back(i);
      const Index m = static_cast<Index>(rest.size());
      std::vector<double> rp(3 * m), fitv(m, 0.0);
      for (Index i = 0; i < m; ++i)
        for (int k = 0; k < 3; ++k) rp[3 * i + k] = pts[3 * rest[i] + k];
      if (mu > 0) {
        DevBuf<double> dc, dw, dq, dout;
        dc.upload(cp);
        dw.upload(weights);
        dq.upload(rp);
        dout.resize(m);
        EvaluateRequest er;
        er.model = &it->model;
        er.centers_dev = dc.data();
        er.mu = mu;
        er.weights_dev = dw.data();
        er.bbox = bbox;
        er.points_dev = dq.data();
        er.m = m;
        er.accuracy = accuracy;
        er.precision = it->precision;
        er.out_dev = dout.data();
        evaluate(er);
        fitv = dout.to_host();
      }
      std::vector<double> res(m);
      for (Index i = 0; i < m; ++i) res[i] = std::fabs(vals[rest[i]] - fitv[i]);
      std::vector<Index> order(m);
      std::iota(order.begin(), order.end(), Index{0});
      std::stable_sort(order.begin(), order.end(), [&](Index a, Index b) { return res[a] < res[b]; });
      Index n_need = 0;
      for (Index i = 0; i < m; ++i)
        if (res[i] >= tolerance) ++n_need;
      if (verbose_out) std::printf("Number of points to fit: %ld\n", static_cast<long>(n_need));
      if (n_need == 0) break;

      // Append the points with the largest residuals that survive the distance filter.
      std::vector<Index> indices(centers);
      for (Index k = m - 1; k >= 0; --k) indices.push_back(rest[order[k]]);
      const auto keep = distance_filter_keep(pts, filtering_distance, indices);
      for (Index k = m - 1; k >= m - n_need; --k) {
        const Index i = rest[order[k]];
        if (keep[i]) {
          centers.push_back(i);
          is_center[i] = 1;
        }
      }
      // Warm start: the old weights, zeros for the new centres, the polynomial part kept.
      const Index mu_new = static_cast<Index>(centers.size());
      std::vector<double> w(mu_new + l, 0.0);
      for (Index i = 0; i < mu; ++i) w[i] = weights[i];
      for (int k = 0; k < l; ++k) w[mu_new + k] = weights[weights.size() - l + k];
      weights = std::move(w);
      filtering_distance = std::max(0.5 * filtering_distance, kMinDistance);
    }

    const Index mu = static_cast<Index>(centers.size());
    std::vector<double> cp(3 * mu);
    for (Index i = 0; i < mu; ++i)
      for (int k = 0; k < 3; ++k) cp[3 * i + k] = pts[3 * centers[i] + k];
    it->weights.upload(weights);
    it->centers.upload(cp);
    it->grad_centers.resize(0);
    it->grad_centers_host.clear();
    it->centers_host = std::move(cp);
    it->mu = mu;
    it->sigma = 0;
    it->bbox = Bbox3::from_host_points(it->centers_host.data(), mu);
    it->fitted = true;
    it->eval_ready = false;
  });
}

// ---- inequality fit (interpolation/inequality_fitter.hpp:43-187) ---------------------------
// values / values_lb / values_ub are NaN where absent. The active-set loop of the reference:
// centres are the equality points plus the active bounds; each round fits them (warm start),
// evaluates at the inequality points, activates violated bounds that survive the distance
// filter (points ordered by their violation, largest first), and deactivates bounds whose
// weight has the wrong sign; it stops when the active set no longer changes.

int pgpu_interpolant_fit_inequality(pgpu_interpolant* it, const double* points, int64_t n,
                                    const double* values, const double* values_lb,
                                    const double* values_ub, double tolerance, int max_iter,
                                    double accuracy) {
  return guarded([&] {
    check_ptr(it, "interpolant");
    check_fit_args(it->model, n, 0, tolerance, INFINITY, max_iter, accuracy, INFINITY);
    check_ptr(points, "points");
    check_ptr(values, "values");
    check_ptr(values_lb, "values_lb");
    check_ptr(values_ub, "values_ub");
    const int l = it->model.l();
    const auto pts = host_copy(points, 3 * n);
    const auto vals = host_copy(values, n);
    const auto lb = host_copy(values_lb, n);
    const auto ub = host_copy(values_ub, n);
    const Bbox3 bbox = Bbox3::from_host_points(pts.data(), n);
    const bool verbose_out = std::getenv("PGPU_VERBOSE") != nullptr;
    constexpr double kMinDistance = 1.0842021724855044e-19;
    double diag = 0;
    for (int k = 0; k < 3; ++k) diag += (bbox.max[k] - bbox.min[k]) * (bbox.max[k] - bbox.min[k]);
    double filtering_distance = std::max(std::sqrt(diag), kMinDistance);

    std::vector<Index> eq, ineq;
    for (Index i = 0; i < n; ++i) {
      if (!std::isnan(vals[i])) eq.push_back(i);
      if (!std::isnan(lb[i]) || !std::isnan(ub[i])) ineq.push_back(i);
    }
    const Index n_ineq = static_cast<Index>(ineq.size());
    std::vector<double> ineq_pts(3 * n_ineq);
    for (Index i = 0; i < n_ineq; ++i)
      for (int k = 0; k < 3; ++k) ineq_pts[3 * i + k] = pts[3 * ineq[i] + k];

    std::vector<double> weights(n + l, 0.0);
    std::set<Index> active_lb, active_ub;
    std::vector<Index> centers;
    std::vector<double> center_weights;
    it->fitted = false;
    while (true) {
      if (verbose_out)
        std::printf("Active lower bounds: %zu, active upper bounds: %zu\n", active_lb.size(),
                    active_ub.size());
      centers = eq;
      std::set_union(active_lb.begin(), active_lb.end(), active_ub.begin(), active_ub.end(),
                     std::back_inserter(centers));
      const Index nc = static_cast<Index>(centers.size());
      std::vector<double> fitv(n_ineq, 0.0);
      if (nc >= l && nc > 0) {
        std::vector<double> cp(3 * nc), cv(nc);
        for (Index i = 0; i < nc; ++i) {
          const Index idx = centers[i];
          for (int k = 0; k < 3; ++k) cp[3 * i + k] = pts[3 * idx + k];
          cv[i] = i < static_cast<Index>(eq.size()) ? vals[idx]
                                                    : (active_lb.count(idx) ? lb[idx] : ub[idx]);
        }
        center_weights.assign(nc + l, 0.0);
        for (Index i = 0; i < nc; ++i) center_weights[i] = weights[centers[i]];
        for (int k = 0; k < l; ++k) center_weights[nc + k] = weights[n + k];
        FitRequest req;
        req.model = &it->model;
        req.points_host = cp.data();
        req.mu = nc;
        req.values_host = cv.data();
        req.tolerance = tolerance;
        req.grad_tolerance = INFINITY;
        req.max_iter = max_iter;
        req.accuracy = accuracy;
        req.grad_accuracy = INFINITY;
        req.initial_weights = center_weights.data();
        req.precision = it->precision;
        req.verbose = verbose_out;
        center_weights = fit(req).weights;
        for (Index i = 0; i < nc; ++i) weights[centers[i]] = center_weights[i];
        for (int k = 0; k < l; ++k) weights[n + k] = center_weights[nc + k];
        if (n_ineq > 0) {
          DevBuf<double> dc, dw, dq, dout;
          dc.upload(cp);
          dw.upload(center_weights);
          dq.upload(ineq_pts);
          dout.resize(n_ineq);
          EvaluateRequest er;
          er.model = &it->model;
          er.centers_dev = dc.data();
          er.mu = nc;
          er.weights_dev = dw.data();
          er.bbox = bbox;
          er.points_dev = dq.data();
          er.m = n_ineq;
          er.accuracy = accuracy;
          er.precision = it->precision;
          er.out_dev = dout.data();
          evaluate(er);
          fitv = dout.to_host();
        }
      } else {
        center_weights.assign(l, 0.0);
      }

      // Violations at the points that are not centres, largest first, through the filter.
      std::vector<char> is_center(n, 0);
      for (Index c : centers) is_center[c] = 1;
      std::vector<double> viol(n, 0.0);
      for (Index i = 0; i < n_ineq; ++i) {
        const Index idx = ineq[i];
        const double lr = std::isnan(lb[idx]) ? 0.0 : std::max(lb[idx] - fitv[i], 0.0);
        const double ur = std::isnan(ub[idx]) ? 0.0 : std::max(fitv[i] - ub[idx], 0.0);
        viol[idx] = std::max(lr, ur);
      }
      std::vector<Index> order;
      for (Index i = 0; i < n; ++i)
        if (!is_center[i]) order.push_back(i);
      std::stable_sort(order.begin(), order.end(), [&](Index a, Index b) { return viol[a] > viol[b]; });
      const auto keep = distance_filter_keep(pts, filtering_distance, order);

      bool changed = false;
      for (Index i = 0; i < n_ineq; ++i) {
        const Index idx = ineq[i];
        if (!std::isnan(lb[idx])) {
          if (active_lb.count(idx)) {
            if (weights[idx] <= 0.0) {
              active_lb.erase(idx);
              changed = true;
            }
          } else if (fitv[i] < lb[idx] - tolerance) {
            if (keep[idx]) {
              active_lb.insert(idx);
              weights[idx] = 0.0;
            }
            changed = true;
          }
        }
        if (!std::isnan(ub[idx])) {
          if (active_ub.count(idx)) {
            if (weights[idx] >= 0.0) {
              active_ub.erase(idx);
              changed = true;
            }
          } else if (fitv[i] > ub[idx] + tolerance) {
            if (keep[idx]) {
              active_ub.insert(idx);
              weights[idx] = 0.0;
            }
            changed = true;
          }
        }
      }
      if (!changed) break;
      filtering_distance = std::max(0.5 * filtering_distance, kMinDistance);
    }

    const Index nc = static_cast<Index>(centers.size());
    std::vector<double> cp(3 * nc);
    for (Index i = 0; i < nc; ++i)
      for (int k = 0; k < 3; ++k) cp[3 * i + k] = pts[3 * centers[i] + k];
    it->weights.upload(center_weights);
    it->centers.upload(cp);
    it->grad_centers.resize(0);
    it->grad_centers_host.clear();
    it->centers_host = std::move(cp);
    it->mu = nc;
    it->sigma = 0;
    it->bbox = Bbox3::from_host_points(it->centers_host.data(), nc);
    it->fitted = true;
    it->eval_ready = false;
  });
}
