/*
 * polatory_gpu.h — C ABI of the GB300 RBF fit/evaluate library (libpolatory_gpu.so).
 *
 * Every entry point returns an int status (PGPU_OK == 0). On failure the message is
 * available from pgpu_last_error() (thread-local). Buffers may be host or device
 * pointers: the library inspects each pointer with cudaPointerGetAttributes and copies
 * host buffers to the device itself. Points are row-major double[n * 3].
 *
 * Reference interfaces replaced (paths inside polatory/polatory):
 *   - pgpu_rbf_*            : include/polatory/rbf/rbf.hpp:11-118, rbf/make_rbf.hpp:24-50
 *   - pgpu_model_*          : include/polatory/model.hpp:23-183
 *   - pgpu_evaluator_*      : include/polatory/fmm/fmm_evaluator.hpp:17-106 and
 *                             include/polatory/fmm/fmm_symmetric_evaluator.hpp:15-86
 *                             (factories src/fmm/make_fmm_evaluator.cpp:40-279)
 *   - pgpu_interpolant_*    : include/polatory/interpolant.hpp:54-218
 *   - pgpu_fit_batch        : no single reference counterpart; it runs Interpolant::fit
 *                             (interpolant.hpp:77-113) over many independent problems.
 *   - pgpu_server_*         : no reference counterpart; serving loop over Interpolant
 *                             fit/evaluate.
 */
#ifndef POLATORY_GPU_H_
#define POLATORY_GPU_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------------------ */
enum {
  PGPU_OK = 0,
  PGPU_INVALID_ARGUMENT = 1, /* std::invalid_argument in the reference */
  PGPU_RUNTIME_ERROR = 2,    /* std::runtime_error in the reference */
  PGPU_CUDA_ERROR = 3,
  PGPU_OUT_OF_MEMORY = 4,
  PGPU_NOT_IMPLEMENTED = 5,
  PGPU_MAX_ITER = 6,         /* "reached the maximum number of iterations" (runtime_error) */
  PGPU_TIMEOUT = 7,          /* a bounded device wait ran out */
  PGPU_REJECTED = 8          /* serving admission refused (HBM budget) */
};

/* ---- RBF kernels (reference short names, rbf/make_rbf.hpp:28-43) --------------------- */
enum {
  PGPU_RBF_BH2 = 0,  /* Biharmonic2D        rbf/polyharmonic_even.hpp */
  PGPU_RBF_BH3 = 1,  /* Biharmonic3D        rbf/polyharmonic_odd.hpp  */
  PGPU_RBF_CUB = 2,  /* CovCubic            rbf/cov_cubic.hpp */
  PGPU_RBF_EXP = 3,  /* CovExponential      rbf/cov_exponential.hpp */
  PGPU_RBF_GAU = 4,  /* CovGaussian         rbf/cov_gaussian.hpp */
  PGPU_RBF_GC3 = 5,  /* CovGeneralizedCauchy3 */
  PGPU_RBF_GC5 = 6,  /* CovGeneralizedCauchy5 */
  PGPU_RBF_GC7 = 7,  /* CovGeneralizedCauchy7 */
  PGPU_RBF_GC9 = 8,  /* CovGeneralizedCauchy9 */
  PGPU_RBF_SPH = 9,  /* CovSpherical */
  PGPU_RBF_SP3 = 10, /* CovSpheroidal3 */
  PGPU_RBF_SP5 = 11, /* CovSpheroidal5 */
  PGPU_RBF_SP7 = 12, /* CovSpheroidal7 */
  PGPU_RBF_SP9 = 13, /* CovSpheroidal9 */
  PGPU_RBF_TH2 = 14, /* Triharmonic2D */
  PGPU_RBF_TH3 = 15, /* Triharmonic3D */
  PGPU_RBF_COUNT = 16
};

#define PGPU_MAX_RBFS 4

/* One RBF: kind, its two parameters (scale/c or psill/range) and the row-major 3x3
 * anisotropy matrix A (the kernel is evaluated at A * (x - y)). */
typedef struct pgpu_rbf {
  int32_t kind;
  int32_t reserved;
  double params[2];
  double aniso[9];
} pgpu_rbf;

/* Model<3>: a sum of RBFs, the polynomial degree (-1 = none .. 2) and the nugget. */
typedef struct pgpu_model {
  int32_t n_rbfs;
  int32_t poly_degree;
  double nugget;
  pgpu_rbf rbfs[PGPU_MAX_RBFS];
} pgpu_model;

/* Arithmetic of the fit/evaluate path. PLAIN: all FP64 (the drop-in). MIXED: FP32 near
 * field and far field with FP64 Krylov, residual recomputation and polynomial block. */
enum { PGPU_PRECISION_PLAIN = 0, PGPU_PRECISION_MIXED = 1 };

/* FMM evaluator flavours (fmm/kernel.hpp, gradient_kernel.hpp, gradient_transpose_kernel.hpp,
 * hessian_kernel.hpp). */
enum {
  PGPU_KERNEL_VALUE = 0,              /* km=1, kn=1 */
  PGPU_KERNEL_GRADIENT = 1,           /* km=3, kn=1 */
  PGPU_KERNEL_GRADIENT_TRANSPOSE = 2, /* km=1, kn=3 */
  PGPU_KERNEL_HESSIAN = 3             /* km=3, kn=3 */
};

/* ---- library ----------------------------------------------------------------------- */
const char* pgpu_last_error(void);
int pgpu_version(void);
/* Selects the CUDA device used by later calls of this thread (default 0). */
int pgpu_set_device(int device);
/* Releases cached device memory held by the library's pool. */
int pgpu_release_cached_memory(void);
/* Phase profiler (no reference counterpart): CUDA events around every instrumented region of
 * the library stream. report writes a JSON object {region: {calls, ms, flops, bytes}} into buf
 * (truncated to size) and synchronizes the stream. launch_count counts kernel launches. */
int pgpu_profile_enable(int on);
int pgpu_profile_reset(void);
int pgpu_profile_report(char* buf, int64_t size);
int pgpu_launch_count(int64_t* out);
/* Host-side fault injection for failure-detection tests (no reference counterpart); nothing
 * here faults the GPU. what = PGPU_INJECT_ALLOC: the `after`-th next device allocation made by
 * this thread (1 = the next one) fails as an exhausted memory pool would, so the running call
 * returns PGPU_OUT_OF_MEMORY. what = PGPU_INJECT_M2L_STALL: in the next tensor-core M2L launch
 * of this thread, the first CTA leaves the operator copy of its first pipeline stage unissued
 * and polls its mbarrier at most `after` times, so that bounded wait runs out: the CTA waits
 * for its other copies in flight and its MMAs, frees its TMEM and returns, and the call returns
 * PGPU_TIMEOUT. after <= 0 clears the injection. */
enum { PGPU_INJECT_ALLOC = 1, PGPU_INJECT_M2L_STALL = 2 };
int pgpu_debug_inject(int what, int64_t after);
/* The process-wide cache of far-field (M2L) operators (no reference counterpart): bytes and
 * entries it holds, and its byte limit. Operators of the homogeneous kernels (bh3, th3) are
 * stored once for every box; other kernels have one entry per cell radius, which follows the
 * bounding box of each point set, so the least recently used entries are dropped past the
 * limit (PGPU_M2L_CACHE_MB in the environment at start-up, 8192 MiB by default). An entry in
 * use by a running evaluation is freed when that evaluation ends. Any pointer may be NULL.
 * pgpu_operator_cache_limit sets the limit in bytes (>= 0) and evicts down to it. */
int pgpu_operator_cache_stats(int64_t* bytes, int64_t* entries, int64_t* limit);
int pgpu_operator_cache_limit(int64_t bytes);
/* Synchronizes the library stream of this thread. */
int pgpu_synchronize(void);
/* The library's CUDA stream of this thread (a cudaStream_t), for event timing by callers. */
int pgpu_stream(void** out);

/* ---- RBF pointwise evaluation (rbf/rbf_base.hpp:40-53) -------------------------------- */
/* Evaluates the anisotropic kernel at n difference vectors (host buffers). Any of values
 * (n), gradients (n*3) or hessians (n*9, row-major) may be NULL. Runs on the host; used to
 * check the device formulas. Kinds without a Hessian (cub, sph) return
 * PGPU_RUNTIME_ERROR when hessians != NULL, as rbf/cov_cubic.hpp:59 throws. */
int pgpu_rbf_evaluate(const pgpu_rbf* rbf, const double* diffs, int64_t n, double* values,
                      double* gradients, double* hessians);
/* cpd_order (rbf_base.hpp:37) and support radius (rbf_base.hpp:97) of a kernel. */
int pgpu_rbf_cpd_order(const pgpu_rbf* rbf, int* out);
int pgpu_rbf_support_radius_isotropic(const pgpu_rbf* rbf, double* out);
/* Model validation: poly_degree within [cpd_order-1, 2] (model.hpp:37-50), nugget >= 0. */
int pgpu_model_validate(const pgpu_model* model);
int pgpu_model_poly_basis_size(const pgpu_model* model, int64_t* out);

/* ---- FMM evaluator (fmm/fmm_evaluator.hpp:17-41, fmm_symmetric_evaluator.hpp:15-37) ---- */
typedef struct pgpu_evaluator pgpu_evaluator;
/* bbox = {minx, miny, minz, maxx, maxy, maxz}. symmetric != 0 selects the symmetric
 * evaluator (sources == targets, set_points). Only VALUE and HESSIAN kinds exist as
 * symmetric evaluators, as in the reference factories. */
int pgpu_evaluator_create(const pgpu_rbf* rbf, int kernel_kind, int symmetric,
                          const double bbox[6], int precision, pgpu_evaluator** out);
int pgpu_evaluator_destroy(pgpu_evaluator* ev);
int pgpu_evaluator_set_accuracy(pgpu_evaluator* ev, double accuracy);
int pgpu_evaluator_set_source_points(pgpu_evaluator* ev, const double* points, int64_t n);
int pgpu_evaluator_set_target_points(pgpu_evaluator* ev, const double* points, int64_t n);
int pgpu_evaluator_set_points(pgpu_evaluator* ev, const double* points, int64_t n);
/* Tuning (no reference counterpart; the reference picks everything from the accuracy):
 * backend 0 = automatic, 1 = exact direct sums, 2 = FMM where the kernel supports it;
 * order = Chebyshev nodes per axis (4, 6 or 8; 0 = from the accuracy); leaf_level = octree
 * depth of the leaves (-1 = automatic). */
int pgpu_evaluator_configure(pgpu_evaluator* ev, int backend, int order, int leaf_level);
/* weights: km * n_sources values in the caller's point order. */
int pgpu_evaluator_set_weights(pgpu_evaluator* ev, const double* weights, int64_t n);
/* out: kn * n_targets values in the caller's target order. */
int pgpu_evaluator_evaluate(pgpu_evaluator* ev, double* out, int64_t n);

/* Allocation-free direct sums (no counterpart in the reference). For callers whose device
 * memory is owned and budgeted by their own allocator, so that the library may not allocate:
 * out[i] = sum_j weights[j] * phi(A (trg_i - src_j)), exact FP64 sums, on the caller's stream
 * (NULL = legacy default stream). All pointers must be device pointers; nothing is allocated or
 * copied. Partial sums live in a fixed 16 MiB device array compiled into the library (held by
 * every GPU that loads it until exit), which limits a call to 2,097,152 targets; larger calls
 * return PGPU_INVALID_ARGUMENT. The entry point runs on the caller's current CUDA device (not the
 * device chosen by pgpu_set_device), and every pointer must be memory of that device or managed
 * memory. The first call on a device looks the array up on that device (make it before any
 * stream capture) and keeps its address until exit: do not call the entry point again after
 * cudaDeviceReset or another teardown of the device's primary context. Calls share the array:
 * calls that may overlap on the GPU race and must be serialised. */
int pgpu_direct_evaluate_noalloc(const pgpu_rbf* rbf, const double* src_points, int64_t n_src,
                                 const double* weights, const double* trg_points, int64_t n_trg,
                                 double* out, void* stream);

/* ---- component tests of the solver and the preconditioner ------------------------------
 * Device runs of the FGMRES and of one RAS domain on caller-given inputs (host buffers), so that
 * the reference's own unit tests of these components can be restated against the device code:
 * test/krylov/test_krylov.cpp:21-137 and test/preconditioner/test_{fine,coarse}_grid.cpp. */
/* FGMRES (src/krylov/fgmres.cpp, gmres.cpp) on the dense row-major n x n operator op, with the
 * optional dense right preconditioner pc and initial solution x0 (NULL: identity / zero), for
 * iters <= n iterations: after iteration k, solutions[k * n ..] receives the solution estimate
 * (Fgmres::solution_vector) and rel_residuals[k] the relative residual estimate
 * (GmresBase::relative_residual). */
int pgpu_krylov_fgmres_dense(int64_t n, const double* op, const double* pc, const double* rhs,
                             const double* x0, int iters, double* solutions, double* rel_residuals);
/* One RAS domain holding all n points (preconditioner/fine_grid.hpp:36-195,
 * coarse_grid.hpp:19-159; value points only): order is a permutation of 0..n-1 whose first l
 * entries are the polynomial points of the Lagrange basis, inner the fine-grid inner flag of each
 * entry of order. coarse != 0 solves rhs (n values) as the coarse grid (use_inverse != 0: through
 * the explicit inverse that a multilevel preconditioner keeps), writing all n weights and the l
 * polynomial coefficients; coarse == 0 solves it as a fine-grid domain, writing the weights of
 * the inner points (zeros elsewhere). precision MIXED uses FP32 factors. out: n + l values. */
int pgpu_ras_domain_solve(const pgpu_model* model, const double* points, int64_t n,
                          const int64_t* order, const unsigned char* inner, int coarse,
                          int use_inverse, int precision, const double* rhs, double* out);

/* ---- Interpolant (interpolant.hpp:54-218) --------------------------------------------- */
typedef struct pgpu_interpolant pgpu_interpolant;

/* Fit statistics of the last fit: FGMRES iterations, final residuals, timings (s). */
typedef struct pgpu_fit_stats {
  int32_t iterations;
  int32_t levels;          /* RAS levels */
  double residual;         /* inf-norm residual at the data points of the accepted fit */
  double grad_residual;
  double setup_seconds;    /* tree + preconditioner setup */
  double solve_seconds;    /* FGMRES loop */
  int64_t n_domains;       /* RAS domains over all fine levels */
  int32_t precision_used;  /* PGPU_PRECISION_* of the arithmetic that produced the weights */
  int32_t fell_back;       /* 1: a MIXED fit met a non-finite FP32 value and reran in FP64 */
} pgpu_fit_stats;

int pgpu_interpolant_create(const pgpu_model* model, pgpu_interpolant** out);
int pgpu_interpolant_destroy(pgpu_interpolant* it);
/* precision: PGPU_PRECISION_PLAIN (default) or PGPU_PRECISION_MIXED. */
int pgpu_interpolant_set_precision(pgpu_interpolant* it, int precision);
/* Interpolant::fit (interpolant.hpp:82-113). grad_points may be NULL when sigma == 0.
 * values: mu + 3 * sigma entries (the values, then the three derivatives of each gradient
 * point). initial may be NULL (warm start otherwise: weights of centres and gradient centres
 * at the same coordinates). Fits with gradient points run in FP64 whatever the precision;
 * kernels without a Hessian (cub, sph) return PGPU_RUNTIME_ERROR with the reference's message. */
int pgpu_interpolant_fit(pgpu_interpolant* it, const double* points, int64_t mu,
                         const double* grad_points, int64_t sigma, const double* values,
                         double tolerance, double grad_tolerance, int max_iter, double accuracy,
                         double grad_accuracy, const pgpu_interpolant* initial);
/* Interpolant::evaluate (interpolant.hpp:58-67). out: m + 3 * mg entries. */
int pgpu_interpolant_evaluate(pgpu_interpolant* it, const double* points, int64_t m,
                              const double* grad_points, int64_t mg, double accuracy,
                              double grad_accuracy, double* out);
/* Interpolant::evaluate_impl (interpolant.hpp:69-75): reuses the evaluator built by the
 * last evaluate / set_evaluation_bbox. */
int pgpu_interpolant_evaluate_impl(pgpu_interpolant* it, const double* points, int64_t m,
                                   const double* grad_points, int64_t mg, double* out);
/* isosurface::RbfFieldFunction::operator() (isosurface/rbf_field_function.hpp:21-23) over the
 * nodes of a lattice (isosurface/rmt/lattice.hpp:421-447, primitive_lattice.hpp:41-43): the
 * node positions (lc_origin + lc) * basis (row vector times the row-major 3 x 3 basis, whose rows
 * are the lattice vectors) are formed on the device from the n integer lattice coordinates lcs
 * (n x 3, host or device), the interpolant is evaluated there through the evaluator of the last
 * set_evaluation_bbox / evaluate (as evaluate_impl), and out (n) receives value - isovalue. */
int pgpu_interpolant_evaluate_lattice(pgpu_interpolant* it, const double lc_origin[3],
                                      const double basis[9], const int32_t* lcs, int64_t n,
                                      double isovalue, double* out);
/* Interpolant::set_evaluation_bbox_impl (interpolant.hpp:201-210). */
int pgpu_interpolant_set_evaluation_bbox(pgpu_interpolant* it, const double bbox[6],
                                         double accuracy, double grad_accuracy);
int pgpu_interpolant_is_fitted(const pgpu_interpolant* it, int* out);
int pgpu_interpolant_num_weights(const pgpu_interpolant* it, int64_t* out);
/* weights layout [lambda (mu), lambda_grad (3 sigma, row-major), c (l)] (interpolant.hpp:88). */
int pgpu_interpolant_weights(const pgpu_interpolant* it, double* out, int64_t n);
int pgpu_interpolant_num_centers(const pgpu_interpolant* it, int64_t* mu, int64_t* sigma);
int pgpu_interpolant_centers(const pgpu_interpolant* it, double* centers, double* grad_centers);
int pgpu_interpolant_bbox(const pgpu_interpolant* it, double bbox[6]);
int pgpu_interpolant_fit_stats(const pgpu_interpolant* it, pgpu_fit_stats* out);
/* Interpolant::fit_incrementally (interpolant.hpp:115-150, interpolation/incremental_fitter.hpp:
 * 46-183): fits a growing subset of the points (largest residuals first, thinned by the
 * reference's distance filter) until every point is within the tolerance; the interpolant's
 * centres are that subset. Gradient points: PGPU_NOT_IMPLEMENTED. */
int pgpu_interpolant_fit_incrementally(pgpu_interpolant* it, const double* points, int64_t mu,
                                       const double* grad_points, int64_t sigma,
                                       const double* values, double tolerance,
                                       double grad_tolerance, int max_iter, double accuracy,
                                       double grad_accuracy);
/* Interpolant::fit_inequality (interpolant.hpp:151-191, interpolation/inequality_fitter.hpp:
 * 43-187): values, values_lb, values_ub of n entries each, NaN where absent; the centres become
 * the equality points plus the active bounds. */
int pgpu_interpolant_fit_inequality(pgpu_interpolant* it, const double* points, int64_t n,
                                    const double* values, const double* values_lb,
                                    const double* values_ub, double tolerance, int max_iter,
                                    double accuracy);
/* Interpolant::save / Interpolant::load (interpolant.hpp:218, POLATORY_IMPLEMENT_LOAD_SAVE,
 * with Write/Read<Interpolant> at interpolant.hpp:345-367): the reference's binary file format,
 * so models move between the two implementations. Errors: "cannot open file '<name>'". */
int pgpu_interpolant_save(const pgpu_interpolant* it, const char* filename);
int pgpu_interpolant_load(const char* filename, pgpu_interpolant** out);

/* ---- batched fits (no single reference counterpart: Interpolant::fit over many problems) --- */
/* One independent fit (+ optional evaluation). Inputs are host or device pointers; outputs are
 * written where the pointers point. status receives the PGPU_* code of this fit. */
typedef struct pgpu_fit_problem {
  const double* points;     /* n x 3 */
  int64_t n;
  const double* values;     /* n */
  double tolerance;
  int32_t max_iter;
  int32_t iterations;       /* out */
  const double* eval_points; /* m x 3, may be NULL */
  int64_t m;
  double* eval_out;         /* m, may be NULL */
  double* weights_out;      /* n + l, may be NULL */
  double residual;          /* out: inf-norm residual at the data points */
  int32_t status;           /* out */
  int32_t reserved;
} pgpu_fit_problem;

/* Fits every problem with the same model. Problems are taken largest first by n_workers host
 * threads (0 = automatic), each with its own CUDA stream, so independent fits overlap on the
 * GPU. Returns PGPU_OK when every problem succeeded, otherwise the first failing status (each
 * problem's own status is in its struct). */
int pgpu_fit_batch(const pgpu_model* model, int precision, pgpu_fit_problem* problems,
                   int64_t n_problems, int n_workers);

/* ---- serving (no reference counterpart) ----------------------------------------------- */
/* A request loop over fit and evaluate requests with continuous batching: requests are
 * admitted in arrival order as worker slots and HBM budget free up (a later request that fits
 * may start before an earlier one that does not); admitted requests run concurrently, each on
 * its worker's CUDA stream. Fitted models stay resident on the device in numbered slots;
 * evaluate requests against a slot wait for that slot's fit. The caller keeps every buffer of a
 * request alive until the request completes. */
typedef struct pgpu_server pgpu_server;

enum { PGPU_REQUEST_FIT = 0, PGPU_REQUEST_EVALUATE = 1 };

typedef struct pgpu_request {
  int32_t kind;          /* PGPU_REQUEST_FIT or PGPU_REQUEST_EVALUATE */
  int32_t slot;          /* model slot written by a fit / read by an evaluation */
  const pgpu_model* model; /* fit only (copied at submit) */
  const double* points;  /* fit: data points; evaluate: query points (n x 3) */
  int64_t n;
  const double* values;  /* fit only */
  double tolerance;      /* fit only */
  int32_t max_iter;      /* fit only */
  int32_t precision;     /* PGPU_PRECISION_* */
  double* out;           /* evaluate: n values */
} pgpu_request;

typedef struct pgpu_server_stats {
  int64_t submitted, completed, failed, rejected, in_flight, queued;
  int64_t bytes_in_use, peak_bytes, budget_bytes;
} pgpu_server_stats;

/* n_workers: concurrent requests (0 = 8); hbm_budget_bytes: admission budget (0 = 150 GB). */
int pgpu_server_create(int n_workers, int64_t hbm_budget_bytes, pgpu_server** out);
int pgpu_server_destroy(pgpu_server* s);
/* Queues a request; returns a ticket. PGPU_REJECTED when its estimated device memory alone
 * exceeds the budget. */
int pgpu_server_submit(pgpu_server* s, const pgpu_request* req, int64_t* ticket);
/* done = 1 once the request has finished; status is its PGPU_* code and latency the seconds
 * from submit to completion. */
int pgpu_server_poll(pgpu_server* s, int64_t ticket, int* done, int* status, double* latency);
int pgpu_server_wait(pgpu_server* s, int64_t ticket, int* status, double* latency);
int pgpu_server_stats_get(pgpu_server* s, pgpu_server_stats* out);
/* Estimated device bytes the server charges against the budget for a request. */
int64_t pgpu_server_estimate_bytes(const pgpu_request* req);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* POLATORY_GPU_H_ */
