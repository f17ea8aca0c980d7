// Mixed-precision factor + FP64 refinement drivers (see mixed_driver.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "gb300solve.h"

namespace gbs {

struct MixedOptions {
  int tier = GBS_TIER_TF32X3;
  double tol = 1e-13;     // normwise backward error to reach
  int max_iter = 30;      // refinement steps before falling back to FP64
};

struct MixedResult {
  int tier = GBS_TIER_TF32X3;   // tier that produced the answer (GBS_TIER_FP64 after a fallback)
  int iterations = 0;
  int fell_back = 0;
  int singular = 0;             // the FP64 factorization met an exactly-zero pivot
  double backward_error = 0.0;
};

int mixed_lu_solve(cudaStream_t s, int n, int nrhs, const double* A, int64_t lda, const double* B, int64_t ldb,
                   double* X, int64_t ldx, const MixedOptions& opt, MixedResult* res);

}  // namespace gbs
