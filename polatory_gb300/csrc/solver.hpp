// Fit and evaluate drivers: Operator (interpolation/operator.hpp:19-127), ResidualEvaluator
// (residual_evaluator.hpp:26-171), FGMRES (src/krylov/{gmres_base,gmres,fgmres}.cpp) and Solver
// (solver.hpp:22-154), with every vector resident on the device.
#pragma once

#include <memory>
#include <vector>

#include "common.hpp"
#include "evaluator.hpp"
#include "model.hpp"

namespace pgpu {

struct FitResult {
  std::vector<double> weights;  // [mu + 3 sigma + l]
  int iterations = 0;
  int levels = 0;
  double residual = 0;
  double grad_residual = 0;
  double setup_seconds = 0;
  double solve_seconds = 0;
  Index n_domains = 0;
  int precision_used = PGPU_PRECISION_PLAIN;  // arithmetic of the solve that produced the weights
  bool fell_back = false;                     // a mixed solve met a non-finite FP32 value
};

struct FitRequest {
  const ModelDesc* model = nullptr;
  const double* points_host = nullptr;  // mu x 3
  Index mu = 0;
  const double* grad_points_host = nullptr;  // sigma x 3
  Index sigma = 0;
  const double* values_host = nullptr;  // mu + 3 sigma
  double tolerance = 0;
  double grad_tolerance = 0;
  int max_iter = 100;
  double accuracy = INFINITY;
  double grad_accuracy = INFINITY;
  const double* initial_weights = nullptr;  // host, mu + 3 sigma + l, or null
  int precision = PGPU_PRECISION_PLAIN;
  bool verbose = false;
  // Internal: the plain solve loop (FP64 operator and residuals) with the preconditioner in the
  // fit's arithmetic type (set by fit() for mixed requests below the mixed-operator threshold).
  bool plain_loop = false;
};

FitResult fit(const FitRequest& req);

struct EvaluateRequest {
  const ModelDesc* model = nullptr;
  const double* centers_dev = nullptr;  // device, mu x 3
  Index mu = 0;
  const double* grad_centers_dev = nullptr;
  Index sigma = 0;
  const double* weights_dev = nullptr;  // device, mu + 3 sigma + l
  Bbox3 bbox;                           // evaluation bbox (query U centres)
  const double* points_dev = nullptr;   // device, m x 3
  Index m = 0;
  const double* grad_points_dev = nullptr;
  Index mg = 0;
  double accuracy = INFINITY;
  double grad_accuracy = INFINITY;
  int precision = PGPU_PRECISION_PLAIN;
  double* out_dev = nullptr;  // m + 3 mg
};

void evaluate(const EvaluateRequest& req);

// Component test of the device FGMRES on a dense n x n operator (host buffers, row-major), with
// an optional dense right preconditioner and initial solution (null: identity / zero): after
// iteration k the solution estimate goes to solutions[k n ..] and the relative residual
// estimate to rel_residuals[k].
void krylov_fgmres_dense(Index n, const double* op, const double* pc, const double* rhs,
                         const double* x0, int iters, double* solutions, double* rel_residuals);

}  // namespace pgpu
