// Batched fits: a pool of host workers, each with its own CUDA stream (the library context is
// per thread), takes independent fit problems largest first; kernels of different fits overlap
// on the GPU. Used by pgpu_fit_batch and by the serving loop.
#include "batch.hpp"

#include <omp.h>

#include <algorithm>
#include <atomic>
#include <numeric>
#include <thread>

#include "solver.hpp"

namespace pgpu {

void set_device(int device);

namespace {

void run_one(const ModelDesc& model, int precision, pgpu_fit_problem& p) {
  std::vector<double> pts(3 * p.n), vals(p.n);
  auto fetch = [](const double* src, double* dst, size_t n) {
    if (n == 0) return;
    if (is_device_pointer(src)) {
      PGPU_CUDA(cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyDeviceToHost, stream()));
      PGPU_CUDA(cudaStreamSynchronize(stream()));
    } else {
      std::copy(src, src + n, dst);
    }
  };
  fetch(p.points, pts.data(), 3 * p.n);
  fetch(p.values, vals.data(), p.n);
  FitRequest req;
  req.model = &model;
  req.points_host = pts.data();
  req.mu = p.n;
  req.values_host = vals.data();
  req.tolerance = p.tolerance;
  req.grad_tolerance = INFINITY;
  req.max_iter = p.max_iter;
  req.precision = precision;
  FitResult r = fit(req);
  p.iterations = r.iterations;
  p.residual = r.residual;
  if (p.weights_out) {
    auto kind = is_device_pointer(p.weights_out) ? cudaMemcpyHostToDevice : cudaMemcpyHostToHost;
    PGPU_CUDA(cudaMemcpyAsync(p.weights_out, r.weights.data(), r.weights.size() * sizeof(double),
                              kind, stream()));
  }
  if (p.m > 0 && p.eval_points && p.eval_out) {
    DevBuf<double> centers, w, q, out;
    centers.upload(pts);
    w.upload(r.weights);
    copy_in(q, p.eval_points, 3 * p.m);
    out.resize(p.m);
    EvaluateRequest er;
    er.model = &model;
    er.centers_dev = centers.data();
    er.mu = p.n;
    er.weights_dev = w.data();
    Bbox3 qb = is_device_pointer(p.eval_points) ? bbox_of_device_points(q.data(), p.m)
                                                : Bbox3::from_host_points(p.eval_points, p.m);
    er.bbox = qb.hull(Bbox3::from_host_points(pts.data(), p.n));
    er.points_dev = q.data();
    er.m = p.m;
    er.precision = precision;
    er.out_dev = out.data();
    evaluate(er);
    copy_out(p.eval_out, out.data(), p.m);
  }
  sync();
}

}  // namespace

int run_batch(const ModelDesc& model, int precision, pgpu_fit_problem* problems, int64_t n,
              int n_workers, int device, std::string* first_error) {
  if (n == 0) return PGPU_OK;
  if (n_workers <= 0) n_workers = static_cast<int>(std::min<int64_t>(n, 16));
  n_workers = static_cast<int>(std::min<int64_t>(n_workers, n));
  std::vector<int64_t> order(n);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(),
                   [&](int64_t a, int64_t b) { return problems[a].n > problems[b].n; });
  std::atomic<int64_t> next{0};
  std::vector<std::string> messages(n);
  auto work = [&] {
    omp_set_num_threads(1);  // the host set-up of each fit runs on its own worker
    try {
      set_device(device);
    } catch (const Error&) {
    }
    while (true) {
      const int64_t k = next.fetch_add(1);
      if (k >= n) break;
      pgpu_fit_problem& p = problems[order[k]];
      try {
        run_one(model, precision, p);
        p.status = PGPU_OK;
      } catch (const Error& e) {
        p.status = e.code;
        messages[order[k]] = e.what();
      } catch (const std::exception& e) {
        p.status = PGPU_RUNTIME_ERROR;
        messages[order[k]] = e.what();
      }
    }
  };
  std::vector<std::thread> pool;
  for (int i = 0; i < n_workers; ++i) pool.emplace_back(work);
  for (auto& t : pool) t.join();
  for (int64_t i = 0; i < n; ++i) {
    if (problems[i].status != PGPU_OK) {
      if (first_error)
        *first_error = "fit " + std::to_string(i) + " of the batch failed: " + messages[i];
      return problems[i].status;
    }
  }
  return PGPU_OK;
}

}  // namespace pgpu
