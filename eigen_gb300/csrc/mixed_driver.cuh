// Mixed-precision factor + FP64 refinement drivers (see mixed_driver.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "gb300solve.h"

namespace gbs {

struct MixedOptions {
  int tier = GBS_TIER_TF32X3;
  int refine = GBS_REFINE_AUTO;  // AUTO: classic for TF32X3, GMRES-IR otherwise
  double tol = 1e-13;            // normwise backward error to reach
  int max_iter = 30;             // outer refinement steps before the FP64 fallback
  int gmres_restart = 40;        // Krylov vectors per GMRES-IR correction
  double gmres_tol = 1e-10;      // relative preconditioned-residual target of one correction
  double shift_factor = 4.0;     // LLT tiers: initial diagonal shift = shift_factor * u_factorization
  int lookahead = 1;             // LU: overlap each block's panels with the previous block's trailing update
  int residual = GBS_RESID_AUTO; // how the FP64 residuals are computed (gbs_residual_mode)
  int pivoting = GBS_PIVOT_AUTO; // LU panels: tournament or the reference's partial pivoting (gbs_pivoting)
};

// R = B - A X (B null: R = A X), FP64-accurate, nrhs columns, on device
// buffers; method: gbs_residual_mode (AUTO: tensor cores from n = 1024).
int residual_device(cudaStream_t s, int n, int nrhs, const double* A, int64_t lda, const double* X, int64_t ldx,
                    const double* B, int64_t ldb, double* R, int64_t ldr, int method);

struct MixedResult {
  int tier = GBS_TIER_TF32X3;    // tier that produced the answer (GBS_TIER_FP64 after a fallback)
  int solver = GBS_REFINE_CLASSIC;
  int iterations = 0;
  int inner_iterations = 0;
  int fell_back = 0;
  int singular = 0;              // FP64 factorization met a zero pivot / non-SPD column
  double backward_error = 0.0;
  double shift = 0.0;
};

int mixed_lu_solve(cudaStream_t s, int n, int nrhs, const double* A, int64_t lda, const double* B, int64_t ldb,
                   double* X, int64_t ldx, const MixedOptions& opt, MixedResult* res);
int mixed_llt_solve(cudaStream_t s, int n, int nrhs, const double* A, int64_t lda, const double* B, int64_t ldb,
                    double* X, int64_t ldx, const MixedOptions& opt, MixedResult* res);
// mixed_lu_solve with A in host memory (column-major, leading dimension lda):
// dA (n x n, leading dimension n) receives it.  For n in [2048, 20480] with up
// to 16 right-hand sides and look-ahead on, A crosses in column chunks that
// the factorization takes in as they land; otherwise in one copy first.  The
// results are identical to mixed_lu_solve's on the same A.  B and X are
// device buffers.
int mixed_lu_solve_host(cudaStream_t s, int n, int nrhs, const double* a, int64_t lda, double* dA, const double* B,
                        int64_t ldb, double* X, int64_t ldx, const MixedOptions& opt, MixedResult* res);
// The chunk plan mixed_lu_solve_host uses for order n (see gbs_streamed_input_plan).
int streamed_input_plan(int n, int cap, int* col, int* iter, int* rolling);

}  // namespace gbs
