// Batched fits over a pool of host workers with per-thread CUDA streams.
#pragma once

#include "common.hpp"
#include "model.hpp"

namespace pgpu {

// Runs every problem; returns PGPU_OK or the first failing status.
int run_batch(const ModelDesc& model, int precision, pgpu_fit_problem* problems, int64_t n,
              int n_workers, int device);

}  // namespace pgpu
