// Serving loop: a queue of fit and evaluate requests drained by a pool of workers, each with
// its own CUDA stream (the library context is per thread), under a device-memory budget.
//
// Admission (continuous batching): whenever a worker is free it takes the first queued request
// that is ready (an evaluation is ready once the fit it reads has finished) and whose charge
// fits in the budget left; a request that does not fit may be passed by later ones at most
// kMaxBypass times, after which admission waits for it. A request's charge is a fixed part plus
// a per-point estimate scaled by the largest ratio of measured peak device bytes to that
// estimate seen so far on large requests of its kind, so the estimate calibrates itself from
// real runs. Fitted models stay resident
// on the device; their bytes count against the budget until a later fit replaces them and no
// queued evaluation still refers to them.
#include <omp.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>

#include "common.hpp"
#include "evaluator.hpp"
#include "model.hpp"
#include "solver.hpp"

namespace pgpu {
void set_device(int device);
}  // namespace pgpu

using namespace pgpu;

namespace {

constexpr int kMaxBypass = 32;

// Per-point device bytes of a request before calibration: fits hold points, values, weights,
// the Krylov basis and the preconditioner's domain matrices (about 350 points per domain,
// up to 1024 points each); evaluations hold the queries, results and far-field expansions.
int64_t per_point_estimate(const pgpu_request& r) {
  if (r.kind == PGPU_REQUEST_FIT) return r.precision == PGPU_PRECISION_MIXED ? 6144 : 12288;
  return 256;
}

// Fixed device bytes of a request: working buffers plus a share for the process-wide cache of
// far-field translation matrices that a new model may grow.
int64_t fixed_estimate(const pgpu_request& r) {
  return r.kind == PGPU_REQUEST_FIT ? (512ll << 20) : (256ll << 20);
}

// Requests this large calibrate the per-point estimate; smaller ones are dominated by the
// fixed part.
constexpr int64_t kCalibrationPoints = 50000;

int64_t base_estimate(const pgpu_request& r) {
  return fixed_estimate(r) + std::max<int64_t>(r.n, 0) * per_point_estimate(r);
}

struct Resident {
  ModelDesc model;
  DevBuf<double> centers, weights;
  Bbox3 bbox;
  Index mu = 0;
  int64_t bytes = 0;
  std::atomic<int64_t>* counter = nullptr;
  ~Resident() {
    if (counter) counter->fetch_sub(bytes);
  }
};

struct Item {
  int64_t ticket = 0;
  pgpu_request req{};
  ModelDesc model;      // fit only
  int64_t dep = -1;     // evaluate: the fit ticket it reads
  int64_t charge = 0;
  int bypassed = 0;
  double t_submit = 0;
};

struct Result {
  bool done = false;
  int status = PGPU_OK;
  double latency = 0;
  std::string message;
};

}  // namespace

struct pgpu_server {
  int device = 0;
  int n_workers = 8;
  int64_t budget = 0;

  std::mutex mu;
  std::condition_variable work_cv, done_cv;
  std::deque<std::unique_ptr<Item>> queue;
  std::unordered_map<int64_t, Result> results;
  std::unordered_map<int32_t, int64_t> slot_last_fit;  // submitted
  std::unordered_map<int32_t, int64_t> slot_current;   // finished
  std::map<int64_t, std::shared_ptr<Resident>> versions;
  std::unordered_map<int64_t, int> version_refs;  // queued evaluations per fit ticket
  std::unordered_map<int64_t, int> fit_status;    // finished fits
  std::atomic<int64_t> resident_bytes{0};
  int64_t in_use = 0, peak = 0, in_flight = 0;
  int64_t next_ticket = 1;
  int64_t submitted = 0, completed = 0, failed = 0, rejected = 0;
  double calib[2] = {1.0, 1.0};  // measured / estimated per-point bytes, per request kind
  bool stop = false;
  std::vector<std::thread> workers;

  int64_t charge_of(const pgpu_request& r) const {
    return fixed_estimate(r) +
           static_cast<int64_t>(static_cast<double>(std::max<int64_t>(r.n, 0)) *
                                static_cast<double>(per_point_estimate(r)) * calib[r.kind]);
  }

  bool fit_finished(int64_t t) const { return fit_status.count(t) != 0; }

  // Drops versions no slot holds and no queued evaluation reads (mu held).
  void collect_versions() {
    for (auto it = versions.begin(); it != versions.end();) {
      const int64_t t = it->first;
      bool current = false;
      for (auto& kv : slot_current)
        if (kv.second == t) current = true;
      auto r = version_refs.find(t);
      if (!current && (r == version_refs.end() || r->second == 0)) {
        version_refs.erase(t);
        it = versions.erase(it);
      } else {
        ++it;
      }
    }
  }

  void finish(const Item& it, int status, const std::string& msg) {
    Result& r = results[it.ticket];
    r.done = true;
    r.status = status;
    r.message = msg;
    r.latency = wall_seconds() - it.t_submit;
    ++completed;
    if (status != PGPU_OK) ++failed;
  }

  // Picks the next request to run, or null (mu held). Fails requests that can never run.
  std::unique_ptr<Item> pick() {
    bool head_blocked = false;
    for (auto q = queue.begin(); q != queue.end();) {
      Item& it = **q;
      if (it.req.kind == PGPU_REQUEST_EVALUATE && !fit_finished(it.dep)) {
        ++q;
        continue;
      }
      if (it.req.kind == PGPU_REQUEST_EVALUATE && fit_status[it.dep] != PGPU_OK) {
        --version_refs[it.dep];
        finish(it, PGPU_INVALID_ARGUMENT, "the fit this evaluation reads failed");
        q = queue.erase(q);
        done_cv.notify_all();
        continue;
      }
      it.charge = charge_of(it.req);
      const int64_t held = in_use + resident_bytes.load();
      if (held + it.charge <= budget) {
        std::unique_ptr<Item> out = std::move(*q);
        queue.erase(q);
        return out;
      }
      if (in_flight == 0) {
        finish(it, PGPU_OUT_OF_MEMORY,
               "request does not fit in the budget left by resident models");
        if (it.req.kind == PGPU_REQUEST_EVALUATE) --version_refs[it.dep];
        q = queue.erase(q);
        done_cv.notify_all();
        continue;
      }
      if (!head_blocked) {
        head_blocked = true;
        if (++it.bypassed > kMaxBypass) return nullptr;
      }
      ++q;
    }
    return nullptr;
  }

  void run_fit(Item& it, int64_t* measured) {
    const pgpu_request& r = it.req;
    std::vector<double> pts(3 * r.n), vals(r.n);
    auto fetch = [](const double* src, double* dst, size_t n) {
      if (n == 0) return;
      if (is_device_pointer(src)) {
        PGPU_CUDA(
            cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyDeviceToHost, stream()));
        PGPU_CUDA(cudaStreamSynchronize(stream()));
      } else {
        std::copy(src, src + n, dst);
      }
    };
    fetch(r.points, pts.data(), 3 * r.n);
    fetch(r.values, vals.data(), r.n);
    FitRequest fr;
    fr.model = &it.model;
    fr.points_host = pts.data();
    fr.mu = r.n;
    fr.values_host = vals.data();
    fr.tolerance = r.tolerance;
    fr.grad_tolerance = INFINITY;
    fr.max_iter = r.max_iter;
    fr.precision = r.precision;
    FitResult res = fit(fr);
    auto m = std::make_shared<Resident>();
    m->model = it.model;
    m->centers.upload(pts);
    m->weights.upload(res.weights);
    m->bbox = Bbox3::from_host_points(pts.data(), r.n);
    m->mu = r.n;
    m->bytes = static_cast<int64_t>((pts.size() + res.weights.size()) * sizeof(double));
    pgpu::sync();
    *measured = thread_device_peak();
    std::lock_guard<std::mutex> lk(mu);
    m->counter = &resident_bytes;
    resident_bytes.fetch_add(m->bytes);
    versions[it.ticket] = std::move(m);
    // Fits on one slot may finish out of order: the slot holds the latest submitted one.
    auto cur = slot_current.find(r.slot);
    if (cur == slot_current.end() || cur->second < it.ticket) slot_current[r.slot] = it.ticket;
  }

  void run_evaluate(Item& it, int64_t* measured) {
    std::shared_ptr<Resident> m;
    {
      std::lock_guard<std::mutex> lk(mu);
      m = versions.at(it.dep);
      --version_refs[it.dep];
    }
    // Other workers may read the model too: if this evaluation throws with launches in flight,
    // they finish before the model's reference is dropped (the last holder frees it).
    struct SyncOnExit {
      ~SyncOnExit() { sync_quiet(); }
    } sync_on_exit;
    const pgpu_request& r = it.req;
    DevBuf<double> q, out;
    copy_in(q, r.points, 3 * r.n);
    out.resize(r.n);
    EvaluateRequest er;
    er.model = &m->model;
    er.centers_dev = m->centers.data();
    er.mu = m->mu;
    er.weights_dev = m->weights.data();
    Bbox3 qb = is_device_pointer(r.points) ? bbox_of_device_points(q.data(), r.n)
                                           : Bbox3::from_host_points(r.points, r.n);
    er.bbox = qb.hull(m->bbox);
    er.points_dev = q.data();
    er.m = r.n;
    er.precision = r.precision;
    er.out_dev = out.data();
    evaluate(er);
    copy_out(r.out, out.data(), r.n);
    *measured = thread_device_peak();
  }

  void worker_main(int omp_threads) {
    omp_set_num_threads(omp_threads);
    bool device_ok = true;
    try {
      set_device(device);
    } catch (const Error&) {
      device_ok = false;
    }
    std::unique_lock<std::mutex> lk(mu);
    while (true) {
      std::unique_ptr<Item> it;
      work_cv.wait(lk, [&] {
        if (!queue.empty()) it = pick();
        return it != nullptr || (stop && queue.empty());
      });
      if (!it) break;
      in_use += it->charge;
      peak = std::max(peak, in_use + resident_bytes.load());
      ++in_flight;
      lk.unlock();

      int status = PGPU_OK;
      std::string msg;
      int64_t measured = 0;
      try {
        if (!device_ok) throw Error(PGPU_CUDA_ERROR, "cannot select the server's device");
        const int64_t base = thread_device_bytes();
        reset_thread_device_peak();
        if (it->req.kind == PGPU_REQUEST_FIT)
          run_fit(*it, &measured);
        else
          run_evaluate(*it, &measured);
        measured -= base;
      } catch (const Error& e) {
        status = e.code;
        msg = e.what();
      } catch (const std::bad_alloc&) {
        status = PGPU_OUT_OF_MEMORY;
        msg = "out of host memory";
      } catch (const std::exception& e) {
        status = PGPU_RUNTIME_ERROR;
        msg = e.what();
      }

      lk.lock();
      in_use -= it->charge;
      --in_flight;
      if (status == PGPU_OK && it->req.n >= kCalibrationPoints) {
        const double ratio = static_cast<double>(measured) /
                             static_cast<double>(it->req.n * per_point_estimate(it->req));
        double& c = calib[it->req.kind];
        c = std::max(c, std::min(ratio, 4.0));
      }
      if (it->req.kind == PGPU_REQUEST_FIT) fit_status[it->ticket] = status;
      finish(*it, status, msg);
      collect_versions();
      work_cv.notify_all();
      done_cv.notify_all();
    }
  }

  void start() {
    const int hw = static_cast<int>(std::max(1u, std::thread::hardware_concurrency()));
    const int omp_threads = std::max(1, hw / n_workers);
    for (int i = 0; i < n_workers; ++i)
      workers.emplace_back([this, omp_threads] { worker_main(omp_threads); });
  }

  // Drains the queue, stops the workers and frees resident models on a worker's device.
  void shutdown() {
    {
      std::lock_guard<std::mutex> lk(mu);
      stop = true;
    }
    work_cv.notify_all();
    for (auto& t : workers) t.join();
    workers.clear();
    std::thread([this] {
      try {
        set_device(device);
        versions.clear();
        pgpu::sync();
      } catch (const Error&) {
      }
    }).join();
  }
};

namespace pgpu {

int server_create(int n_workers, int64_t budget, pgpu_server** out) {
  auto s = std::make_unique<pgpu_server>();
  PGPU_CUDA(cudaGetDevice(&s->device));
  s->n_workers = n_workers > 0 ? n_workers : 8;
  s->budget = budget > 0 ? budget : (150ll << 30);
  s->start();
  *out = s.release();
  return PGPU_OK;
}

void server_destroy(pgpu_server* s) {
  s->shutdown();
  delete s;
}

int64_t server_estimate(const pgpu_request& r) { return base_estimate(r); }

void server_submit(pgpu_server* s, const pgpu_request& r, int64_t* ticket) {
  auto it = std::make_unique<Item>();
  it->req = r;
  if (r.kind == PGPU_REQUEST_FIT) it->model = model_from_c(r.model);
  it->t_submit = wall_seconds();
  std::lock_guard<std::mutex> lk(s->mu);
  if (s->stop) throw Error(PGPU_INVALID_ARGUMENT, "server is shutting down");
  if (base_estimate(r) > s->budget) {
    ++s->rejected;
    throw Error(PGPU_REJECTED, "request needs more device memory than the server's budget");
  }
  if (r.kind == PGPU_REQUEST_EVALUATE) {
    auto f = s->slot_last_fit.find(r.slot);
    if (f == s->slot_last_fit.end())
      throw Error(PGPU_INVALID_ARGUMENT, "slot holds no model");
    it->dep = f->second;
    ++s->version_refs[it->dep];
  }
  it->ticket = s->next_ticket++;
  if (r.kind == PGPU_REQUEST_FIT) s->slot_last_fit[r.slot] = it->ticket;
  s->results[it->ticket] = Result{};
  ++s->submitted;
  *ticket = it->ticket;
  s->queue.push_back(std::move(it));
  s->work_cv.notify_one();
}

// Reports a ticket; a finished ticket's record is released once reported.
bool server_poll(pgpu_server* s, int64_t ticket, bool block, int* status, double* latency,
                 std::string* msg) {
  std::unique_lock<std::mutex> lk(s->mu);
  auto r = s->results.find(ticket);
  if (r == s->results.end()) throw Error(PGPU_INVALID_ARGUMENT, "unknown or already reported ticket");
  if (block) s->done_cv.wait(lk, [&] { return s->results[ticket].done; });
  Result& res = s->results[ticket];
  if (!res.done) return false;
  *status = res.status;
  *latency = res.latency;
  *msg = res.message;
  s->results.erase(ticket);
  return true;
}

void server_stats(pgpu_server* s, pgpu_server_stats* o) {
  std::lock_guard<std::mutex> lk(s->mu);
  o->submitted = s->submitted;
  o->completed = s->completed;
  o->failed = s->failed;
  o->rejected = s->rejected;
  o->in_flight = s->in_flight;
  o->queued = static_cast<int64_t>(s->queue.size());
  o->bytes_in_use = s->in_use + s->resident_bytes.load();
  o->peak_bytes = s->peak;
  o->budget_bytes = s->budget;
}

}  // namespace pgpu
