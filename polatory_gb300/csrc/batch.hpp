// Batched fits over a pool of host workers with per-thread CUDA streams.
#pragma once

#include <string>

#include "common.hpp"
#include "model.hpp"

namespace pgpu {

// Runs every problem; returns PGPU_OK or the status of the first failing problem (in problem
// order), whose index and message go to *first_error.
int run_batch(const ModelDesc& model, int precision, pgpu_fit_problem* problems, int64_t n,
              int n_workers, int device, std::string* first_error);

}  // namespace pgpu
